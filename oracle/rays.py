"""FP64 restatement of the paraxial ray chain (oracle; test infrastructure only).

Follows, operation by operation:
  - ``Ray``                          ray.py:8-166
  - ``FreeSpaceParaxial.propagate``  propagator.py:51-72
  - ``FreeSpaceDirCosine.propagate`` propagator.py:79-116
  - ``run_iter`` / ``run_to_end``    run.py:47-116 (a propagator is inserted
    before EVERY component, with per-ray distance ``component.z - ray.z``)
  - components                       components.py:137-559
  - ``AberratedLensKrivanek``        components.py:177-215 with
    ``W_krivanek`` / ``grad_W_krivanek`` aberrations.py:42-108 (polar form,
    atan2 / hypot / cos(m phi) exactly as written there); its Jacobian for the
    ABCD by central differences of that gradient
  - ``custom_jacobian_matrix``       utils.py:7-43 (rows/cols x, y, dx, dy, _one)
  - ``solve_model``                  run.py:150-179
  - ``accumulate_matrices``          transfer.py:126-147 (M_last @ ... @ M_0)

All arithmetic is NumPy float64 (or complex128 when a caller differentiates
by complex step).  The ``aperture`` component has no reference counterpart
(the reference has no Aperture component); it is this project's extension:
rays with (x-cx)^2 + (y-cy)^2 >= r^2 are marked blocked and otherwise pass
unchanged.
"""
from __future__ import annotations

import numpy as np


class ORay:
    """Structure-of-arrays ray record (ray.py:39-45).  Fields are arrays."""

    __slots__ = ("x", "y", "dx", "dy", "z", "pathlength", "one", "alive")

    def __init__(self, x, y, dx, dy, z=0.0, pathlength=0.0, one=1.0, alive=None):
        self.x = np.asarray(x)
        self.y = np.asarray(y)
        self.dx = np.asarray(dx)
        self.dy = np.asarray(dy)
        self.z = np.asarray(z)
        self.pathlength = np.asarray(pathlength)
        self.one = np.asarray(one)
        self.alive = alive  # None == all rays pass (reference behaviour)

    def copy(self, **kw):
        d = {k: getattr(self, k) for k in self.__slots__}
        d.update(kw)
        return ORay(**d)

    @staticmethod
    def from_f32(x, y, dx, dy, z=0.0, pathlength=0.0):
        """Promote float32 ray state to float64 exactly (the GPU's inputs)."""
        f = lambda a: np.asarray(a, dtype=np.float32).astype(np.float64)  # noqa: E731
        return ORay(f(x), f(y), f(dx), f(dy), np.asarray(z, np.float64),
                    np.asarray(pathlength, np.float64))


def propagate(r: ORay, d) -> ORay:
    """propagator.py:64-72: x += dx*d, y += dy*d, z += d, pathlength += d."""
    return r.copy(x=r.x + r.dx * d, y=r.y + r.dy * d, z=r.z + d,
                  pathlength=r.pathlength + d)


def propagate_dircos(r: ORay, d) -> ORay:
    """propagator.py:100-110 (FreeSpaceDirCosine): N = sqrt(1 + dx^2 + dy^2),
    L = dx/N, M = dy/N; x += L/N*d, y += M/N*d, z = z*_one + d,
    pathlength += d*N."""
    n = np.sqrt(1 + r.dx ** 2 + r.dy ** 2)
    L = r.dx / n
    M = r.dy / n
    return r.copy(x=r.x + L / n * d, y=r.y + M / n * d, z=r.z * r.one + d,
                  pathlength=r.pathlength + d * n)


def _prop(propagator):
    if propagator in (None, "paraxial"):
        return propagate
    if propagator == "dircos":
        return propagate_dircos
    raise ValueError(propagator)


def comp_z(c: dict):
    """Axial position used by run_iter (ThickLens.z is z_po, components.py:448-452)."""
    if c["kind"] == "thicklens":
        return c["z_po"]
    return c["z"]


def _descan_terms(c: dict):
    """Descanner offsets (components.py:320-372) plus this project's tilt columns.

    The reference adds, per output coordinate, a linear function of scan
    position minus the scan position/tilt itself.  The optional keys
    ``pxo_sxi .. syo_syi`` (d out / d scan tilt) default to 0, which is the
    reference's behaviour.
    """
    de = dict(c.get("descan_error", {}))
    g = lambda k: de.get(k, 0.0)  # noqa: E731
    spx, spy = c["scan_pos_x"], c["scan_pos_y"]
    stx, sty = c.get("scan_tilt_x", 0.0), c.get("scan_tilt_y", 0.0)
    ax = spx * g("pxo_pxi") + spy * g("pxo_pyi") + g("offpxi") - spx
    ay = spx * g("pyo_pxi") + spy * g("pyo_pyi") + g("offpyi") - spy
    adx = spx * g("sxo_pxi") + spy * g("sxo_pyi") + g("offsxi") - stx
    ady = spx * g("syo_pxi") + spy * g("syo_pyi") + g("offsyi") - sty
    if any(k in de for k in ("pxo_sxi", "pxo_syi", "pyo_sxi", "pyo_syi",
                             "sxo_sxi", "sxo_syi", "syo_sxi", "syo_syi")):
        ax = ax + stx * g("pxo_sxi") + sty * g("pxo_syi")
        ay = ay + stx * g("pyo_sxi") + sty * g("pyo_syi")
        adx = adx + stx * g("sxo_sxi") + sty * g("sxo_syi")
        ady = ady + stx * g("syo_sxi") + sty * g("syo_syi")
    return ax, ay, adx, ady


def apply_component(c: dict, r: ORay) -> ORay:
    """One component's ``__call__`` (components.py), same operation order."""
    k = c["kind"]
    if k in ("plane", "detector", "scangrid", "source"):
        return r  # components.py:133, 248, 405; source.py:20-34
    if k == "lens":  # components.py:161-174
        f = c["focal_length"]
        x, y, dx, dy = r.x, r.y, r.dx, r.dy
        return r.copy(dx=-x / f + dx, dy=-y / f + dy,
                      pathlength=r.pathlength - (x ** 2 + y ** 2) / (2 * f),
                      one=r.one * 1.0)
    if k == "thicklens":  # components.py:431-446
        f = c["focal_length"]
        x, y, dx, dy = r.x, r.y, r.dx, r.dy
        return r.copy(dx=-x / f + dx, dy=-y / f + dy,
                      pathlength=r.pathlength - (x ** 2 + y ** 2) / (2 * f),
                      z=r.z - (c["z_po"] - c["z_pi"]), one=r.one * 1.0)
    if k == "scanner":  # components.py:279-285
        return r.copy(x=r.x + c["scan_pos_x"] * r.one,
                      y=r.y + c["scan_pos_y"] * r.one,
                      dx=r.dx + c.get("scan_tilt_x", 0.0) * r.one,
                      dy=r.dy + c.get("scan_tilt_y", 0.0) * r.one)
    if k == "descanner":  # components.py:346-372
        ax, ay, adx, ady = _descan_terms(c)
        return r.copy(x=r.x + ax * r.one, y=r.y + ay * r.one,
                      dx=r.dx + adx * r.one, dy=r.dy + ady * r.one)
    if k == "deflector":  # components.py:476-482 (pathlength uses incoming slopes)
        x, y, dx, dy = r.x, r.y, r.dx, r.dy
        return r.copy(dx=dx + c["def_x"] * r.one, dy=dy + c["def_y"] * r.one,
                      pathlength=r.pathlength + dx * x + dy * y)
    if k == "biprism":  # components.py:553-559 (offset/rotation/side unused)
        x, y, dx, dy = r.x, r.y, r.dx, r.dy
        sgn = np.sign(np.real(x))
        return r.copy(dx=dx + c.get("def_x", 0.0) * r.one * sgn, dy=dy,
                      pathlength=r.pathlength + dx * x + dy * y)
    if k == "rotator":  # components.py:503-523
        a = np.deg2rad(c["angle"]) if not np.iscomplexobj(c["angle"]) else c["angle"] * np.pi / 180
        ca, sa = np.cos(a), np.sin(a)
        return r.copy(x=r.x * ca - r.y * sa, y=r.x * sa + r.y * ca,
                      dx=r.dx * ca - r.dy * sa, dy=r.dx * sa + r.dy * ca)
    if k == "aperture":  # project extension: blocks rays outside the radius
        cx, cy = c.get("centre", (0.0, 0.0))
        rr = (np.real(r.x) - cx) ** 2 + (np.real(r.y) - cy) ** 2
        ok = rr < c["radius"] ** 2
        alive = ok if r.alive is None else (r.alive & ok)
        return r.copy(alive=alive)
    if k == "aberrated_lens":  # components.py:193-215
        f = c["focal_length"]
        x, y, dx, dy = r.x, r.y, r.dx, r.dy
        ideal_dx = -x / f + dx
        ideal_dy = -y / f + dy
        alpha = np.hypot(ideal_dx, ideal_dy)
        phi = np.arctan2(ideal_dy, ideal_dx)
        dwx, dwy = grad_w_krivanek(ideal_dx, ideal_dy, c.get("coeffs", {}))
        return r.copy(dx=ideal_dx + (-dwx / f), dy=ideal_dy + (-dwy / f),
                      pathlength=r.pathlength - (x ** 2 + y ** 2) / (2 * f)
                      + w_krivanek(alpha, phi, c.get("coeffs", {})) / f,
                      one=r.one * 1.0)
    raise NotImplementedError(k)


# ---------------------------------------------------------------- aberrations
_KRIV = ("C10", "C12", "phi12", "C21", "phi21", "C23", "phi23", "C30", "C32", "phi32", "C34",
         "phi34", "C41", "phi41", "C43", "phi43", "C45", "phi45", "C50", "C52", "phi52", "C54",
         "phi54", "C56", "phi56")


def _kc(p: dict):
    return {n: float(p.get(n, 0.0)) for n in _KRIV}


def _brackets(phi, p):
    """aberrations.py:42-48."""
    c = lambda m, ph0: np.cos(m * (phi - ph0))  # noqa: E731
    B2 = p["C10"] + p["C12"] * c(2, p["phi12"])
    B3 = p["C21"] * c(1, p["phi21"]) + p["C23"] * c(3, p["phi23"])
    B4 = p["C30"] + p["C32"] * c(2, p["phi32"]) + p["C34"] * c(4, p["phi34"])
    B5 = p["C41"] * c(1, p["phi41"]) + p["C43"] * c(3, p["phi43"]) + p["C45"] * c(5, p["phi45"])
    B6 = p["C50"] + p["C52"] * c(2, p["phi52"]) + p["C54"] * c(4, p["phi54"]) + p["C56"] * c(6, p["phi56"])
    return B2, B3, B4, B5, B6


def w_krivanek(alpha, phi, coeffs):
    """aberrations.py:51-61."""
    p = _kc(coeffs)
    B2, B3, B4, B5, B6 = _brackets(phi, p)
    a = alpha
    a2 = a * a
    a3 = a2 * a
    a4 = a2 * a2
    a6 = a3 * a3
    return 0.5 * a2 * B2 + (a3 / 3.0) * B3 + 0.25 * a4 * B4 + 0.2 * a4 * a * B5 + (a6 / 6.0) * B6


def grad_w_krivanek(ax, ay, coeffs):
    """aberrations.py:64-108 (polar chain rule, alpha = 0 guarded)."""
    p = _kc(coeffs)
    a = np.hypot(ax, ay)
    phi = np.arctan2(ay, ax)
    B2, B3, B4, B5, B6 = _brackets(phi, p)
    s = lambda m, ph0: np.sin(m * (phi - ph0))  # noqa: E731
    a2 = a * a
    a3 = a2 * a
    a4 = a2 * a2
    a5 = a4 * a
    a6 = a3 * a3
    dwda = a * B2 + a2 * B3 + a3 * B4 + a4 * B5 + a5 * B6
    dwdphi = (0.5 * a2) * (-2.0 * p["C12"] * s(2, p["phi12"]))
    dwdphi += (a3 / 3.0) * (-1.0 * p["C21"] * s(1, p["phi21"]) - 3.0 * p["C23"] * s(3, p["phi23"]))
    dwdphi += (0.25 * a4) * (-2.0 * p["C32"] * s(2, p["phi32"]) - 4.0 * p["C34"] * s(4, p["phi34"]))
    dwdphi += (0.2 * a4 * a) * (-1.0 * p["C41"] * s(1, p["phi41"]) - 3.0 * p["C43"] * s(3, p["phi43"])
                                - 5.0 * p["C45"] * s(5, p["phi45"]))
    dwdphi += (a6 / 6.0) * (-2.0 * p["C52"] * s(2, p["phi52"]) - 4.0 * p["C54"] * s(4, p["phi54"])
                            - 6.0 * p["C56"] * s(6, p["phi56"]))
    a_safe = np.where(a == 0, 1e-30, a)
    inv_a = 1.0 / a_safe
    inv_a2 = inv_a * inv_a
    return (dwda * (ax * inv_a) + dwdphi * (-ay * inv_a2),
            dwda * (ay * inv_a) + dwdphi * (ax * inv_a2))


def aberrated_lens_matrix(c: dict, x, y, dx, dy):
    """5x5 Jacobian of the aberrated lens at one ray state: the Hessian of W
    at the ideal slopes by central differences of grad_w_krivanek (step 1e-6
    of the slope scale); no _one column (the aberration does not scale with
    _one)."""
    f = c["focal_length"]
    ux, uy = -x / f + dx, -y / f + dy
    h = 1e-6 * max(abs(ux), abs(uy), 1e-3)
    gxp, gyp = grad_w_krivanek(ux + h, uy, c.get("coeffs", {}))
    gxm, gym = grad_w_krivanek(ux - h, uy, c.get("coeffs", {}))
    hxx, hyx = (gxp - gxm) / (2 * h), (gyp - gym) / (2 * h)
    gxp, gyp = grad_w_krivanek(ux, uy + h, c.get("coeffs", {}))
    gxm, gym = grad_w_krivanek(ux, uy - h, c.get("coeffs", {}))
    hxy, hyy = (gxp - gxm) / (2 * h), (gyp - gym) / (2 * h)
    hs = 0.5 * (hxy + hyx)
    k = 1.0 / f
    m = np.eye(5)
    m[2, 0], m[2, 1], m[2, 2], m[2, 3] = -k + hxx * k * k, hs * k * k, 1 - hxx * k, -hs * k
    m[3, 0], m[3, 1], m[3, 2], m[3, 3] = hs * k * k, -k + hyy * k * k, -hs * k, 1 - hyy * k
    return m


def run_iter(r: ORay, model, propagator="paraxial"):
    """run.py:75-82: yields (step, ray) for the propagator then the component."""
    prop = _prop(propagator)
    for c in model:
        d = comp_z(c) - r.z
        r = prop(r, d)
        yield ("propagator", d), r
        r = apply_component(c, r)
        yield c, r


def run_to_end(r: ORay, model, propagator="paraxial") -> ORay:
    """run.py:85-116."""
    for _, r in run_iter(r, model, propagator):
        pass
    return r


# ---------------------------------------------------------------- ABCD matrices

def _eye5():
    return np.eye(5, dtype=np.float64)


def free_matrix(d):
    """Jacobian of propagate (tests/test_rays.py:82-103)."""
    m = _eye5()
    m[0, 2] = d
    m[1, 3] = d
    return m


def component_matrix(c: dict, x_at_component=0.0):
    """5x5 Jacobian of one component w.r.t. (x, y, dx, dy, _one) (utils.py:7-43).

    ``x_at_component`` is the central ray's x at the component; only the
    biprism depends on it (d dx / d _one = def_x * sign(x)).
    """
    k = c["kind"]
    m = _eye5()
    if k in ("plane", "detector", "scangrid", "source", "aperture"):
        return m
    if k in ("lens", "thicklens"):
        f = c["focal_length"]
        m[2, 0] = -1.0 / f
        m[3, 1] = -1.0 / f
        return m
    if k == "scanner":
        m[0, 4] = c["scan_pos_x"]
        m[1, 4] = c["scan_pos_y"]
        m[2, 4] = c.get("scan_tilt_x", 0.0)
        m[3, 4] = c.get("scan_tilt_y", 0.0)
        return m
    if k == "descanner":
        m[0:4, 4] = _descan_terms(c)
        return m
    if k == "deflector":
        m[2, 4] = c["def_x"]
        m[3, 4] = c["def_y"]
        return m
    if k == "biprism":
        m[2, 4] = c.get("def_x", 0.0) * np.sign(x_at_component)
        return m
    if k == "rotator":
        a = np.deg2rad(c["angle"])
        ca, sa = np.cos(a), np.sin(a)
        m[0, 0], m[0, 1], m[1, 0], m[1, 1] = ca, -sa, sa, ca
        m[2, 2], m[2, 3], m[3, 2], m[3, 3] = ca, -sa, sa, ca
        return m
    raise NotImplementedError(k)


def dircos_matrix(r: ORay, d):
    """5x5 Jacobian of propagate_dircos at a scalar ray, by complex step
    (exact to rounding) on x, y, dx, dy."""
    m = _eye5()
    h = 1e-30
    base = [complex(float(np.asarray(v).ravel()[0])) for v in (r.x, r.y, r.dx, r.dy)]
    for j in range(4):
        v = list(base)
        v[j] += 1j * h
        o = propagate_dircos(ORay(*[np.array([a]) for a in v], z=0.0, pathlength=0.0), d)
        for i, f in enumerate((o.x, o.y, o.dx, o.dy)):
            m[i, j] = np.imag(f[0]) / h
    return m


def solve_model(r: ORay, model, propagator="paraxial"):
    """run.py:150-179: per-step 5x5 matrices (propagator, component, ...)."""
    prop = _prop(propagator)
    mats = []
    for c in model:
        d = comp_z(c) - r.z
        dd = float(np.asarray(d).ravel()[0])
        mats.append(free_matrix(dd) if prop is propagate else dircos_matrix(r, dd))
        r = prop(r, d)
        if c["kind"] == "aberrated_lens":
            v = [float(np.asarray(t).ravel()[0]) for t in (r.x, r.y, r.dx, r.dy)]
            mats.append(aberrated_lens_matrix(c, *v))
        else:
            mats.append(component_matrix(c, float(np.asarray(r.x).ravel()[0])))
        r = apply_component(c, r)
    return np.array(mats)


def accumulate_matrices(mats):
    """transfer.py:126-147: mats[-1] @ ... @ mats[0]."""
    total = mats[-1]
    for tm in reversed(mats[:-1]):
        total = total @ tm
    return total


def model_abcd(r: ORay, model, propagator="paraxial"):
    """Whole-model ABCD about a scalar central ray (jacobian of run_to_end)."""
    return accumulate_matrices(list(solve_model(r, model, propagator)))

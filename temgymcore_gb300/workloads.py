"""Seeded synthetic workloads with the shapes of the benchmark configurations.

Each generator returns plain NumPy inputs plus a model description as a list
of dicts (``{"kind": ..., <reference field names>}``); ``build_model`` turns
that description into this package's components.  No dataset is read: the
reference publishes no benchmark data, so inputs are drawn from the stated
distributions with ``numpy.random.default_rng(seed)``.
"""
from __future__ import annotations

import numpy as np

from . import components as K

_KIND = {"lens": K.Lens, "plane": K.Plane, "detector": K.Detector, "scangrid": K.ScanGrid,
         "scanner": K.Scanner, "descanner": K.Descanner, "deflector": K.Deflector,
         "biprism": K.Biprism, "rotator": K.Rotator, "thicklens": K.ThickLens,
         "aperture": K.Aperture, "source": K.PointSource, "aberrated_lens": K.AberratedLensKrivanek}


def build_model(spec):
    """List of dict descriptions -> list of components."""
    out = []
    for c in spec:
        kw = {k: v for k, v in c.items() if k != "kind"}
        cls = _KIND[c["kind"]]
        if c["kind"] == "descanner" and "descan_error" in kw:
            kw["descan_error"] = K.DescanError(**kw["descan_error"])
        if c["kind"] in ("detector", "scangrid"):
            kw["pixel_size"] = tuple(kw["pixel_size"])
            kw["shape"] = tuple(int(v) for v in kw["shape"])
            if "centre" in kw:
                kw["centre"] = tuple(kw["centre"])
        if c["kind"] == "source":
            kw = {"z": kw["z"]}
        out.append(cls(**kw))
    return out


def plain_trace(seed: int = 0, n: int = 65536):
    """Plain paraxial trace: N float32 rays, x, y ~ U(-1e-3, 1e-3) m,
    dx, dy ~ N(0, 1e-3) rad, z = 0, pathlength = 0; Lens(z=0.5, f=0.2) then
    Detector(z=1.0, pixel 1e-5 m, 256 x 256)."""
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1e-3, 1e-3, n).astype(np.float32)
    y = rng.uniform(-1e-3, 1e-3, n).astype(np.float32)
    dx = rng.normal(0.0, 1e-3, n).astype(np.float32)
    dy = rng.normal(0.0, 1e-3, n).astype(np.float32)
    spec = [{"kind": "lens", "z": 0.5, "focal_length": 0.2},
            {"kind": "detector", "z": 1.0, "pixel_size": (1e-5, 1e-5), "shape": (256, 256)}]
    return {"x": x, "y": y, "dx": dx, "dy": dy, "z": 0.0, "pathlength": 0.0, "model": spec}


def stem_4d(seed: int = 0, scan=(64, 64), rays_per_probe: int = 1024, scan_step: float = 1e-9,
            defocus: float = 1e-6, camera_length: float = 0.1, det_px: float = 5.5e-5,
            det_shape=(256, 256), semi_conv: float = 5e-3):
    """4D-STEM shadow-image model.

    A point source at z = 0 emits one bundle of ``rays_per_probe`` rays with
    slopes dx, dy ~ U(-semi_conv, semi_conv) rad (shared by every probe, as a
    fixed PointSource sampling is); the sample plane sits ``defocus`` below it
    and carries a ScanGrid (``scan`` positions, step ``scan_step``, rotation
    U(0, 360) degrees), the Scanner and the Descanner; the detector is
    ``camera_length`` further down.  The descan matrix is I + N(0, 1e-3)
    (rows x, y, dx, dy; columns scan x, y, tilt x, tilt y).
    """
    rng = np.random.default_rng(seed)
    dxs = rng.uniform(-semi_conv, semi_conv, rays_per_probe).astype(np.float32)
    dys = rng.uniform(-semi_conv, semi_conv, rays_per_probe).astype(np.float32)
    rot_deg = float(rng.uniform(0.0, 2 * np.pi) * 180.0 / np.pi)
    descan = np.eye(4) + rng.normal(0.0, 1e-3, (4, 4))
    z_s = defocus
    spec_scan = {"kind": "scangrid", "z": z_s, "pixel_size": (scan_step, scan_step),
                 "shape": tuple(scan), "rotation": rot_deg}
    det = {"kind": "detector", "z": z_s + camera_length, "pixel_size": (det_px, det_px),
           "shape": tuple(det_shape)}
    return {"x": np.zeros(rays_per_probe, np.float32), "y": np.zeros(rays_per_probe, np.float32),
            "dx": dxs, "dy": dys, "z": 0.0, "pathlength": 0.0,
            "scangrid": spec_scan, "descan": descan, "detector": det,
            "source_z": 0.0}


def descan_error_from_matrix(m) -> dict:
    m = np.asarray(m)
    if not np.iscomplexobj(m):  # complex entries pass through (complex-step derivatives)
        m = m.astype(np.float64)
    return {"pxo_pxi": m[0, 0], "pxo_pyi": m[0, 1], "pyo_pxi": m[1, 0], "pyo_pyi": m[1, 1],
            "sxo_pxi": m[2, 0], "sxo_pyi": m[2, 1], "syo_pxi": m[3, 0], "syo_pyi": m[3, 1],
            "pxo_sxi": m[0, 2], "pxo_syi": m[0, 3], "pyo_sxi": m[1, 2], "pyo_syi": m[1, 3],
            "sxo_sxi": m[2, 2], "sxo_syi": m[2, 3], "syo_sxi": m[3, 2], "syo_syi": m[3, 3]}


def stem_probe_model(w: dict, spx: float, spy: float):
    """Per-probe model description of ``stem_4d`` at one scan position."""
    z = w["scangrid"]["z"]
    err = descan_error_from_matrix(w["descan"])
    return [{"kind": "source", "z": w["source_z"]},
            dict(w["scangrid"]),
            {"kind": "scanner", "z": z, "scan_pos_x": spx, "scan_pos_y": spy},
            {"kind": "descanner", "z": z, "scan_pos_x": spx, "scan_pos_y": spy,
             "descan_error": err},
            dict(w["detector"])]


def stem_model(w: dict):
    """Components of ``stem_4d`` (scan positions are supplied per probe)."""
    _d = descan_error_from_matrix
    sg = w["scangrid"]
    z = sg["z"]
    return [K.PointSource(z=w["source_z"]),
            K.ScanGrid(z=z, pixel_size=tuple(sg["pixel_size"]), shape=tuple(sg["shape"]),
                       rotation=sg["rotation"]),
            K.Scanner(z=z, scan_pos_x=0.0, scan_pos_y=0.0),
            K.Descanner(z=z, scan_pos_x=0.0, scan_pos_y=0.0,
                        descan_error=K.DescanError(**_d(w["descan"]))),
            K.Detector(z=w["detector"]["z"], pixel_size=tuple(w["detector"]["pixel_size"]),
                       shape=tuple(w["detector"]["shape"]))]


def beamlet_field(seed: int = 0, n_beams: int = 16384, det_shape=(512, 512), det_px: float = 1e-5,
                  aperture_radius: float = 5e-8, waist: float = 1e-9, wavelength: float = 1.97e-12,
                  focal_length: float = 0.5, astigmatic: bool = False):
    """Gaussian-beamlet field (aperture-diffraction geometry).

    ``n_beams`` beamlets sit on a golden-angle spiral filling a circular
    aperture of ``aperture_radius`` at z = 0 (parallel beam, slopes 0),
    waist ``waist``, flat wavefront; amplitudes |a| ~ U(0.5, 1) with phase
    U(0, 2 pi) (complex64); pathlengths 1 m + N(0, 1e-6) m; wavelength
    1.97 pm (200 keV).  Model: Lens(z=f, f) then Detector(z=2f) - the back
    focal plane, where the field is the aperture's diffraction pattern.
    ``astigmatic``: waist_y = waist * U(0.5, 1.5) and theta ~ U(0, pi).
    """
    from .gaussian import fibonacci_spiral
    rng = np.random.default_rng(seed)
    x, y = fibonacci_spiral(n_beams, aperture_radius, alpha=0)
    amp = (rng.uniform(0.5, 1.0, n_beams) * np.exp(1j * rng.uniform(0, 2 * np.pi, n_beams))
           ).astype(np.complex64)
    pl = 1.0 + rng.normal(0.0, 1e-6, n_beams)
    wxy = np.full((n_beams, 2), waist)
    theta = np.zeros(n_beams)
    if astigmatic:
        wxy[:, 1] = waist * rng.uniform(0.5, 1.5, n_beams)
        theta = rng.uniform(0.0, np.pi, n_beams)
    rays = {"x": x, "y": y, "dx": np.zeros(n_beams), "dy": np.zeros(n_beams), "z": 0.0,
            "pathlength": pl, "amplitude": amp, "waist_xy": wxy,
            "radii_of_curv": np.full((n_beams, 2), np.inf), "wavelength": wavelength,
            "theta": theta}
    spec = [{"kind": "lens", "z": focal_length, "focal_length": focal_length},
            {"kind": "detector", "z": 2 * focal_length, "pixel_size": (det_px, det_px),
             "shape": tuple(det_shape)}]
    return {"rays": rays, "model": spec}


def input_field(seed: int = 0, n_beams: int = 16384, grid_shape=(512, 512), px: float = 1e-5,
                wavelength: float = 500e-9, astigmatic: bool = False):
    """Input-plane beamlet field (an image decomposed into Gaussians, the use
    of evaluate_gaussian_input_image, gaussian.py:372-427).

    ``n_beams`` beams on a golden-angle spiral filling a disc of 0.4 of the
    grid half-width; waist = the mean beam spacing (so neighbours overlap),
    flat wavefront; slopes N(0, 1e-4) rad; amplitudes |a| ~ U(0.5, 1), phase
    U(0, 2 pi); pathlength N(0, 1e-6) m; wavelength 500 nm.  Grid: a detector
    of ``grid_shape`` pixels of ``px`` m at z = 0.  ``astigmatic``: waist_y =
    waist * U(0.5, 1.5), theta ~ U(0, pi).
    """
    from .gaussian import fibonacci_spiral
    rng = np.random.default_rng(seed)
    radius = 0.4 * 0.5 * min(grid_shape) * px
    x, y = fibonacci_spiral(n_beams, radius, alpha=0)
    waist = float(np.sqrt(np.pi * radius ** 2 / n_beams))
    amp = (rng.uniform(0.5, 1.0, n_beams) * np.exp(1j * rng.uniform(0, 2 * np.pi, n_beams))
           ).astype(np.complex64)
    wxy = np.full((n_beams, 2), waist)
    theta = np.zeros(n_beams)
    if astigmatic:
        wxy[:, 1] = waist * rng.uniform(0.5, 1.5, n_beams)
        theta = rng.uniform(0.0, np.pi, n_beams)
    rays = {"x": x, "y": y, "dx": rng.normal(0.0, 1e-4, n_beams), "dy": rng.normal(0.0, 1e-4, n_beams),
            "z": 0.0, "pathlength": rng.normal(0.0, 1e-6, n_beams), "amplitude": amp, "waist_xy": wxy,
            "radii_of_curv": np.full((n_beams, 2), np.inf), "wavelength": wavelength, "theta": theta}
    grid = {"kind": "detector", "z": 0.0, "pixel_size": (px, px), "shape": tuple(grid_shape)}
    return {"rays": rays, "grid": grid, "waist": waist}


def gaussian_rays(d: dict):
    """GaussianRay from a ``beamlet_field`` ray dict."""
    from .ray import GaussianRay
    return GaussianRay(x=d["x"], y=d["y"], dx=d["dx"], dy=d["dy"], z=d["z"],
                       pathlength=d["pathlength"], amplitude=d["amplitude"],
                       waist_xy=d["waist_xy"], radii_of_curv=d["radii_of_curv"],
                       wavelength=d["wavelength"], theta=d["theta"])


def stem_fit(seed: int = 0, scan=(32, 32), rays_per_probe: int = 1024, rel_sigma: float = 0.01):
    """Adjoint-fit workload in the plain-trace geometry.

    Bundle at z = 0 with the plain-trace distributions (x, y ~ U(+-1e-3) m,
    dx, dy ~ N(0, 1e-3) rad); scan/descan plane at z = defocus = 0.05 m
    (32 x 32 scan, step 1e-5 m, rotation 37 deg, descan I + N(0, 1e-3));
    Lens(f = 0.2 m) at z = 0.5 m (gap 0.45 m after the scan plane); detector
    at z = 1.0 m (camera length 0.95 m from the scan plane).  The target
    parameters are the nominal ones perturbed by N(0, rel_sigma) relative.
    """
    rng = np.random.default_rng(seed)
    n = rays_per_probe
    x = rng.uniform(-1e-3, 1e-3, n).astype(np.float32)
    y = rng.uniform(-1e-3, 1e-3, n).astype(np.float32)
    dx = rng.normal(0.0, 1e-3, n).astype(np.float32)
    dy = rng.normal(0.0, 1e-3, n).astype(np.float32)
    descan = np.eye(4) + rng.normal(0.0, 1e-3, (4, 4))
    theta0 = np.concatenate([[0.2, 0.05, 0.95, 37.0, 1e-5], descan.reshape(16)])
    theta_true = theta0 * (1.0 + rng.normal(0.0, rel_sigma, theta0.size))
    return {"x": x, "y": y, "dx": dx, "dy": dy, "rows": scan[0], "cols": scan[1], "gap": 0.45,
            "theta0": theta0, "theta_true": theta_true}


def stem_fit_probe_spec(w: dict, theta, p: int):
    """Model description (oracle form) of ``stem_fit`` at probe p for theta."""
    th = np.asarray(theta)
    f, dfc, cl, rot, step = th[:5]
    m = th[5:].reshape(4, 4)
    rows, cols = w["rows"], w["cols"]
    sg = {"kind": "scangrid", "z": dfc, "pixel_size": (step, step), "shape": (rows, cols),
          "rotation": rot}
    return sg, [{"kind": "source", "z": 0.0}, sg,
                {"kind": "scanner", "z": dfc, "scan_pos_x": None, "scan_pos_y": None},
                {"kind": "descanner", "z": dfc, "scan_pos_x": None, "scan_pos_y": None,
                 "descan_error": descan_error_from_matrix(m)},
                {"kind": "lens", "z": dfc + w["gap"], "focal_length": f},
                {"kind": "detector", "z": dfc + cl, "pixel_size": (1e-5, 1e-5), "shape": (256, 256)}]


def batched_sweep(seed: int = 0, n_models: int = 512, n_components=(2, 12),
                  rays=(1e3, 2.6e5)):
    """Batched sweep: n_models independent models with U{2..12} components
    drawn from lens / deflector / biprism / aperture (log-uniform f in
    [0.01, 1] m, spacings U(0.01, 0.1) m), ray counts log-uniform in
    [1e3, 2.6e5] (~2.4e7 rays at 512 models); plain-trace ray distributions;
    targets N(0, 1e-3) m for the adjoint's squared-residual loss."""
    rng = np.random.default_rng(seed)
    specs = []
    for _ in range(n_models):
        nc = int(rng.integers(n_components[0], n_components[1] + 1))
        z = 0.0
        comps = []
        for _ in range(nc):
            z += float(rng.uniform(0.01, 0.1))
            kind = ("lens", "deflector", "biprism", "aperture")[int(rng.integers(0, 4))]
            if kind == "lens":
                comps.append({"kind": "lens", "z": z, "focal_length": float(10 ** rng.uniform(-2, 0))})
            elif kind == "deflector":
                comps.append({"kind": "deflector", "z": z, "def_x": float(rng.normal(0, 1e-3)),
                              "def_y": float(rng.normal(0, 1e-3))})
            elif kind == "biprism":
                comps.append({"kind": "biprism", "z": z, "def_x": float(rng.normal(0, 1e-3))})
            else:
                comps.append({"kind": "aperture", "z": z, "radius": float(rng.uniform(5e-4, 5e-3))})
        specs.append(comps)
    counts = np.round(10 ** rng.uniform(np.log10(rays[0]), np.log10(rays[1]), n_models)).astype(np.int64)
    total = int(counts.sum())
    x = rng.uniform(-1e-3, 1e-3, total).astype(np.float32)
    y = rng.uniform(-1e-3, 1e-3, total).astype(np.float32)
    dx = rng.normal(0.0, 1e-3, total).astype(np.float32)
    dy = rng.normal(0.0, 1e-3, total).astype(np.float32)
    tx = rng.normal(0.0, 1e-3, total).astype(np.float32)
    ty = rng.normal(0.0, 1e-3, total).astype(np.float32)
    return {"specs": specs, "counts": counts, "x": x, "y": y, "dx": dx, "dy": dy, "tx": tx, "ty": ty}

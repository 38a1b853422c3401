"""FP64 restatement of the Gaussian-beamlet detector field (oracle; tests only).

Follows:
  - ``GaussianRay.q_inv`` / ``Q_inv``            gaussian.py:138-177
    (Q_inv = R(theta) diag(1/q) R(theta)^T via the einsum at gaussian.py:221-222)
  - ``Qinv_ABCD``                                gaussian.py:92-96
  - ``zR``, ``w_z``, ``R``, ``q_inv(z, w0, wl)``, ``gaussian_beam``
                                                 gaussian.py:13-32, 99-109
  - ``make_gaussian_image``                      gaussian.py:225-273
  - ``_beam_field``                              gaussian.py:276-316
  - ``propagate_misaligned_gaussian_jax_scan``   gaussian.py:319-337
  - ``map_reduce`` (a plain sum over beams)      gaussian.py:340-369
  - ``decompose_Q_inv``                          gaussian.py:35-89
  - ``evaluate_gaussian_input_image``            gaussian.py:372-400
  - ``_input_beam_field``                        gaussian.py:403-409
  - ``fibonacci_spiral``                         utils.py:297-325
  - ``FresnelPropagator`` / ``fresnel_lens_imaging_solution`` (the
    transfer-function Fresnel method the reference's tests check the
    beamlet field against)                      utils.py:245-272

2x2 inverses are written out explicitly (the reference calls
jnp.linalg.solve); singular matrices give inf/nan which are zeroed with
nan_to_num exactly where the reference zeroes them (B^-1 and Q1, gaussian.py
:283-287) and left alone elsewhere.

``phase_mode``:
  * ``"exact"``  - k*pathlength reduced exactly mod 2*pi (oracle.phase); the
    checker for every phase claim.
  * ``"literal"`` - the reference's literal float64 ``phase + k*pl``.
"""
from __future__ import annotations

import numpy as np

from .grid import grid_coords
from .phase import phase_offset_exact
from .rays import (ORay, aberrated_lens_matrix, apply_component, comp_z, component_matrix,  # noqa: F401
                   free_matrix, propagate)


def q_inv(waist_xy, radii, wavelength):
    """gaussian.py:138-158: per-axis 1/q."""
    wx, wy = waist_xy[..., 0], waist_xy[..., 1]
    rx, ry = radii[..., 0], radii[..., 1]
    wl = wavelength
    with np.errstate(divide="ignore", invalid="ignore"):
        qx = np.where(np.isinf(rx), 1j * wl / (np.pi * wx ** 2), -1.0 / rx + 1j * wl / (np.pi * wx ** 2))
        qy = np.where(np.isinf(ry), 1j * wl / (np.pi * wy ** 2), -1.0 / ry + 1j * wl / (np.pi * wy ** 2))
    return qx, qy


def Q_inv(waist_xy, radii, wavelength, theta):
    """gaussian.py:160-177: R diag(qx, qy) R^T with R = [[c, -s], [s, c]]."""
    qx, qy = q_inv(waist_xy, radii, wavelength)
    n = qx.shape[0]
    d = np.zeros((n, 2, 2), dtype=np.complex128)
    d[:, 0, 0] = qx
    d[:, 1, 1] = qy
    c, s = np.cos(theta), np.sin(theta)
    r = np.zeros((n, 2, 2))
    r[:, 0, 0], r[:, 0, 1], r[:, 1, 0], r[:, 1, 1] = c, -s, s, c
    return np.einsum("nij,njk,npk->nip", r, d, r)


def inv2(m):
    """Explicit batched 2x2 inverse (inf/nan for singular input)."""
    a, b, c, d = m[..., 0, 0], m[..., 0, 1], m[..., 1, 0], m[..., 1, 1]
    with np.errstate(divide="ignore", invalid="ignore"):
        det = a * d - b * c
        out = np.empty_like(m, dtype=np.result_type(m, np.float64))
        out[..., 0, 0] = d / det
        out[..., 0, 1] = -b / det
        out[..., 1, 0] = -c / det
        out[..., 1, 1] = a / det
    return out


def Qinv_ABCD(q1, A, B, C, D):
    """gaussian.py:92-96: solve(A + B Q1, C + D Q1)."""
    return inv2(A + B @ q1) @ (C + D @ q1)


def zR(w0, wavelength):
    """gaussian.py:17-18: Rayleigh range pi w0^2 / wavelength."""
    return (np.pi * np.asarray(w0, np.float64) ** 2) / wavelength


def w_z(w0, z, z_r):
    """gaussian.py:13-14: beam radius at distance z from the waist."""
    return w0 * np.sqrt(1 + (np.asarray(z, np.float64) / z_r) ** 2)


def R_of_z(z, z_r):
    """gaussian.py:21-28: wavefront radius z (1 + (z_r / z)^2); infinite for
    |z| < 1e-10 (elementwise here; the reference's lax.cond takes a scalar)."""
    z = np.asarray(z, np.float64)
    focus = np.abs(z) < 1e-10
    with np.errstate(divide="ignore", invalid="ignore"):
        ratio = np.where(focus, 0.0, z_r / np.where(focus, 1.0, z))
        return np.where(focus, np.inf, z * (1 + ratio ** 2))


def q_inv_z(z, w0, wl):
    """gaussian.py:99-109: 1/q of a beam of waist w0 at distance z."""
    z_r = zR(w0, wl)
    focus = np.abs(np.asarray(z, np.float64)) < 1e-10
    wz = w_z(w0, z, z_r)
    r = R_of_z(z, z_r)
    with np.errstate(divide="ignore"):
        return np.where(focus, 1j * wl / (np.pi * np.asarray(w0, np.float64) ** 2),
                        -(1.0 / r) + 1j * wl / (np.pi * wz ** 2))


def gaussian_beam(x, y, q, k, offset_x=0, offset_y=0):
    """gaussian.py:31-32: exp(1j k ((x + ox)^2 + (y + oy)^2) / 2 q)."""
    return np.exp(1j * k * ((np.asarray(x, np.float64) + offset_x) ** 2 + (y + offset_y) ** 2) / 2 * q)


def beam_abcd(x, y, dx, dy, z, model):
    """Per-beam 5x5 ABCD = jacobian(run_to_end) at each central ray (gaussian.py:234-249)."""
    n = np.asarray(x).size
    r = ORay(np.asarray(x, np.float64).ravel(), np.asarray(y, np.float64).ravel(),
             np.asarray(dx, np.float64).ravel(), np.asarray(dy, np.float64).ravel(),
             np.broadcast_to(np.asarray(z, np.float64), (n,)).copy(), np.zeros(n))
    total = np.broadcast_to(np.eye(5), (n, 5, 5)).copy()
    for c in model:
        d = comp_z(c) - r.z
        fm = np.broadcast_to(np.eye(5), (n, 5, 5)).copy()
        fm[:, 0, 2] = d
        fm[:, 1, 3] = d
        total = fm @ total
        r = propagate(r, d)
        if c["kind"] == "biprism":
            cm = np.broadcast_to(np.eye(5), (n, 5, 5)).copy()
            cm[:, 2, 4] = c.get("def_x", 0.0) * np.sign(r.x)
        elif c["kind"] == "aberrated_lens":
            cm = np.stack([aberrated_lens_matrix(c, r.x[i], r.y[i], r.dx[i], r.dy[i]) for i in range(n)])
        else:
            cm = np.broadcast_to(component_matrix(c), (n, 5, 5))
        total = cm @ total
        r = apply_component(c, r)
    return total


def beam_field_pixels(amp, phase_offset, q1inv, q2inv, r1m, theta1m, A, B, e, f, k, r2,
                      po_exact=None):
    """gaussian.py:276-316 for a chunk of beams (leading axis) over pixels r2 (P, 2).

    Returns (nb, P) complex128.  ``po_exact`` (nb,), if given, replaces the
    literal float64 ``phase_offset`` (the exact-reduced oracle).
    """
    eye = np.eye(2)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        binv = np.nan_to_num(inv2(B), nan=0.0, posinf=0.0, neginf=0.0)
        q1 = np.nan_to_num(inv2(q1inv), nan=0.0, posinf=0.0, neginf=0.0)
        s = r2[None, :, :] - e[:, None, :]  # (nb, P, 2)
        r2m = np.einsum("nij,nj->ni", A, r1m) + np.einsum("nij,nj->ni", B, theta1m)
        denom = A + B @ q1inv
        det = denom[:, 0, 0] * denom[:, 1, 1] - denom[:, 0, 1] * denom[:, 1, 0]
        pref = amp / np.sqrt(det.astype(np.complex128))
        abinv = A @ binv
        phi1 = (np.einsum("ni,nij,nj->n", r1m, abinv, r1m)[:, None]
                - 2 * np.einsum("ni,nij,npj->np", r1m, binv, s))
        aq1 = A @ q1
        b_over = inv2(B @ (aq1 + B))
        p = q1 @ b_over
        phi2 = (np.einsum("ni,nij,nj->n", r2m, p, r2m)[:, None]
                - 2 * np.einsum("ni,nij,npj->np", r2m, p, s))
        q2t = np.einsum("npi,nij,npj->np", s, q2inv, s)
        f_off = 2 * np.einsum("npi,ni->np", s, f)
        phase = (k[:, None] / 2) * (q2t + phi1 - phi2 + f_off)
        if po_exact is None:
            return pref[:, None] * np.exp(1j * (phase + phase_offset[:, None]))
        return pref[:, None] * np.exp(1j * phase) * np.exp(1j * po_exact[:, None])


def make_gaussian_image(rays: dict, model, pixel_index=None, chunk=64, phase_mode="exact"):
    """gaussian.py:225-273.  ``rays`` keys: x, y, dx, dy, z, pathlength,
    amplitude (complex), waist_xy (B,2), radii_of_curv (B,2), wavelength (B,),
    theta (B,).  Returns the (H, W) complex128 field, or the flat pixels
    ``pixel_index`` only when given."""
    grid = model[-1]
    assert grid["kind"] == "detector"
    x = np.asarray(rays["x"], np.float64).ravel()
    n = x.size
    bc = lambda v: np.broadcast_to(np.asarray(v, np.float64), (n,)).copy()  # noqa: E731
    y, dx, dy = bc(rays["y"]), bc(rays["dx"]), bc(rays["dy"])
    z, pl = bc(rays["z"]), bc(rays["pathlength"])
    wl = bc(rays["wavelength"])
    theta = bc(rays["theta"])
    amp = np.broadcast_to(np.asarray(rays["amplitude"], np.complex128), (n,)).copy()
    waist = np.broadcast_to(np.asarray(rays["waist_xy"], np.float64), (n, 2))
    radii = np.broadcast_to(np.asarray(rays["radii_of_curv"], np.float64), (n, 2))

    abcd = beam_abcd(x, y, dx, dy, z, model)
    A, B, C, D = abcd[:, 0:2, 0:2], abcd[:, 0:2, 2:4], abcd[:, 2:4, 0:2], abcd[:, 2:4, 2:4]
    e, f = abcd[:, 0:2, 4], abcd[:, 2:4, 4]
    q1inv = Q_inv(waist, radii, wl, theta)
    q2inv = Qinv_ABCD(q1inv, A, B, C, D)
    r2 = grid_coords(grid)
    if pixel_index is not None:
        r2 = r2[np.asarray(pixel_index).ravel()]
    k = 2 * np.pi / wl
    phase_offset = k * pl
    po = phase_offset_exact(k, pl) if phase_mode == "exact" else None
    r1m = np.stack([x, y], -1)
    t1m = np.stack([dx, dy], -1)
    acc = np.zeros(r2.shape[0], dtype=np.complex128)
    for s in range(0, n, chunk):
        sl = slice(s, s + chunk)
        acc += beam_field_pixels(amp[sl], phase_offset[sl], q1inv[sl], q2inv[sl], r1m[sl],
                                 t1m[sl], A[sl], B[sl], e[sl], f[sl], k[sl], r2,
                                 None if po is None else po[sl]).sum(0)
    if pixel_index is not None:
        return acc
    return acc.reshape(grid["shape"])


def _beams(rays: dict):
    x = np.asarray(rays["x"], np.float64).ravel()
    n = x.size
    bc = lambda v: np.broadcast_to(np.asarray(v, np.float64), (n,)).copy()  # noqa: E731
    return dict(
        x=x, y=bc(rays["y"]), dx=bc(rays["dx"]), dy=bc(rays["dy"]), pl=bc(rays["pathlength"]),
        wl=bc(rays["wavelength"]), theta=bc(rays["theta"]),
        amp=np.broadcast_to(np.asarray(rays["amplitude"], np.complex128), (n,)).copy(),
        waist=np.broadcast_to(np.asarray(rays["waist_xy"], np.float64), (n, 2)),
        radii=np.broadcast_to(np.asarray(rays["radii_of_curv"], np.float64), (n, 2)), n=n)


def input_beam_field_pixels(amp, q1inv, r1m, t1m, k, r1, po):
    """gaussian.py:403-409 for a chunk of beams over pixels r1 (P, 2):
    a * exp(i (k/2) (d^T Q1 d + 2 d.t1m)) * exp(i p), d = r1 - r1m."""
    d = r1[None, :, :] - r1m[:, None, :]
    quad = np.einsum("npi,nij,npj->np", d, q1inv, d)
    tilt = 2 * np.einsum("npi,ni->np", d, t1m)
    phase = (k[:, None] / 2) * (quad + tilt)
    return amp[:, None] * np.exp(1j * phase) * np.exp(1j * po[:, None])


def evaluate_gaussian_input_image(rays: dict, grid: dict, pixel_index=None, chunk=64,
                                  phase_mode="exact"):
    """gaussian.py:372-400: the beams' field in their own plane sampled on
    ``grid`` (no model).  Same ``rays`` keys and ``phase_mode`` as
    ``make_gaussian_image``."""
    b = _beams(rays)
    q1inv = Q_inv(b["waist"], b["radii"], b["wl"], b["theta"])
    r1 = grid_coords(grid)
    if pixel_index is not None:
        r1 = r1[np.asarray(pixel_index).ravel()]
    k = 2 * np.pi / b["wl"]
    po = phase_offset_exact(k, b["pl"]) if phase_mode == "exact" else k * b["pl"]
    r1m = np.stack([b["x"], b["y"]], -1)
    t1m = np.stack([b["dx"], b["dy"]], -1)
    acc = np.zeros(r1.shape[0], dtype=np.complex128)
    for s in range(0, b["n"], chunk):
        sl = slice(s, s + chunk)
        acc += input_beam_field_pixels(b["amp"][sl], q1inv[sl], r1m[sl], t1m[sl], k[sl], r1,
                                       po[sl]).sum(0)
    if pixel_index is not None:
        return acc
    return acc.reshape(grid["shape"])


def decompose_Q_inv(Q_inv, wavelength, eps=1e-12):
    """gaussian.py:35-89 with NumPy's eigh (LAPACK's eigenvector signs)."""
    Q = np.asarray(Q_inv)
    S = np.imag(Q)
    S = 0.5 * (S + np.swapaxes(S, -1, -2))
    _, evecs = np.linalg.eigh(S)
    det = np.linalg.det(evecs)
    sign = np.where(det < 0, -1.0, 1.0)
    evecs = evecs.copy()
    evecs[..., :, 1] *= sign[..., None]
    Vt = np.swapaxes(evecs, -1, -2)
    Qd = Vt @ Q @ evecs
    qdiag = np.stack([Qd[..., 0, 0], Qd[..., 1, 1]], axis=-1)
    imd_pre = np.imag(qdiag)
    with np.errstate(divide="ignore"):
        waists_pre = np.sqrt(np.where(np.abs(imd_pre) > eps, np.abs(wavelength / (np.pi * imd_pre)), np.inf))
    swap = waists_pre[..., 0] < waists_pre[..., 1]
    qdiag = np.where(swap[..., None], qdiag[..., ::-1], qdiag)
    evecs = np.where(swap[..., None, None], evecs[..., :, ::-1], evecs)
    det = np.linalg.det(evecs)
    sign = np.where(det < 0, -1.0, 1.0)
    evecs = evecs.copy()
    evecs[..., :, 1] *= sign[..., None]
    imd, red = np.imag(qdiag), np.real(qdiag)
    with np.errstate(divide="ignore"):
        waists = np.sqrt(np.where(np.abs(imd) > eps, np.abs(wavelength / (np.pi * imd)), np.inf))
        radii = np.where(np.abs(red) > eps, 1.0 / red, np.inf)
    e1 = evecs[..., :, 0]
    theta = np.arctan2(e1[..., 1], e1[..., 0])
    return waists[..., 0], waists[..., 1], radii[..., 0], radii[..., 1], theta


def fibonacci_spiral(nb_samples: int, radius: float, alpha=2):
    """utils.py:297-325 (Vogel / golden-angle spiral in a disc)."""
    ga = np.pi * (3.0 - np.sqrt(5.0))
    np_boundary = np.round(alpha * np.sqrt(nb_samples))
    ii = np.arange(nb_samples)
    rr = np.where(ii > nb_samples - (np_boundary + 1), radius,
                  radius * np.sqrt((ii + 0.5) / (nb_samples - 0.5 * (np_boundary + 1))))
    rr[0] = 0.0
    phi = ii * ga
    return rr * np.cos(phi), rr * np.sin(phi)


def fresnel_tf(u1, side, wavelength, z):
    """utils.py:245-262: Fresnel propagation over z by the transfer-function
    method on a square grid of physical side ``side``: U2 = IFFT(H FFT(u1)),
    H = exp(-i pi wavelength z (fx^2 + fy^2)) (no exp(ikz) factor)."""
    m, n = u1.shape
    dx = side / m
    fx = np.fft.fftfreq(n, d=dx)
    fy = np.fft.fftfreq(m, d=dx)
    FX, FY = np.meshgrid(fx, fy)
    return np.fft.ifft2(np.exp(-1j * np.pi * wavelength * z * (FX ** 2 + FY ** 2)) * np.fft.fft2(u1))


def fresnel_thin_lens(u0, X, Y, pixel, wavelength, z1, f, z2):
    """utils.py:265-272: propagate z1, thin-lens phase exp(-i k r^2 / 2f),
    propagate z2."""
    k = 2 * np.pi / wavelength
    side = u0.shape[0] * pixel
    u = fresnel_tf(u0, side, wavelength, z1)
    u = u * np.exp((-1j * k) / (2 * f) * (X ** 2 + Y ** 2))
    return fresnel_tf(u, side, wavelength, z2)

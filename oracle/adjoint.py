"""FP64 value-and-gradient of the squared-residual loss over a ray chain
(oracle; test infrastructure only).

The reference differentiates with ``jax.value_and_grad`` of a loss over
``run_to_end`` (run.py:85-116; README.md:113-160): reverse-mode AD that
records the forward values and walks the steps backwards.  This module does
the same by hand in NumPy float64 for the paraxial chain:

  loss = sum over alive rays of (x_out - tx)^2 + (y_out - ty)^2

``value_and_raw`` returns the loss and the per-step sums the GPU adjoints
report (one row of 4 per compiled step: the propagator before each component,
then the component), i.e. the loss's derivative with respect to

  propagator            its distance d                       (row[0])
  lens / thicklens      focal_length                         (row[0])
  deflector             def_x, def_y                         (row[0], row[1])
  biprism               def_x                                (row[0])
  scanner / descanner   the shift added to x, y, dx, dy      (row[0..3])
  rotator               the angle in radians                 (row[0])

The steps and their derivatives follow the forward formulas of
propagator.py:64-72 and components.py:161-174, 279-285, 346-372, 476-482,
503-523, 553-559 (restated in ``oracle.rays``).  A biprism's sign and an
aperture's test have zero derivative (as under jax.grad).  ``margins``
reports, per ray, how close each such discrete decision came to flipping,
so a comparison can set aside rays whose decision rounding may flip.
"""
from __future__ import annotations

import numpy as np

from .rays import ORay, _descan_terms, apply_component, comp_z, propagate


def _shift_terms(c):
    if c["kind"] == "scanner":
        return (c["scan_pos_x"], c["scan_pos_y"], c.get("scan_tilt_x", 0.0), c.get("scan_tilt_y", 0.0))
    return _descan_terms(c)


def forward_tape(r: ORay, model):
    """run_iter (run.py:75-82) keeping the state entering every step."""
    tape = []
    for c in model:
        d = comp_z(c) - r.z
        tape.append(("free", d, r))
        r = propagate(r, d)
        tape.append((c, None, r))
        r = apply_component(c, r)
    return tape, r


def value_and_raw(model, x, y, dx, dy, tx, ty, z=0.0):
    """(loss, raw [2 * n_components, 4], output ORay) in float64."""
    r0 = ORay(*(np.asarray(v, np.float64) for v in (x, y, dx, dy)), z=np.asarray(z, np.float64),
              pathlength=np.asarray(0.0))
    tape, out = forward_tape(r0, model)
    alive = np.ones(np.shape(out.x), bool) if out.alive is None else out.alive
    rx = np.where(alive, out.x - np.asarray(tx, np.float64), 0.0)
    ry = np.where(alive, out.y - np.asarray(ty, np.float64), 0.0)
    loss = float(np.sum(rx * rx + ry * ry))
    lx, ly = 2.0 * rx, 2.0 * ry
    ldx = np.zeros_like(lx)
    ldy = np.zeros_like(lx)
    raw = np.zeros((len(tape), 4))
    for s in range(len(tape) - 1, -1, -1):
        step, d, r = tape[s]  # r: the state entering step s
        if step == "free":
            raw[s, 0] = np.sum(lx * r.dx + ly * r.dy)
            ldx = ldx + lx * d
            ldy = ldy + ly * d
            continue
        k = step["kind"]
        if k in ("lens", "thicklens"):
            f = step["focal_length"]
            raw[s, 0] = np.sum(ldx * r.x + ldy * r.y) / (f * f)
            lx = lx - ldx / f
            ly = ly - ldy / f
        elif k == "deflector":
            raw[s, 0] = np.sum(ldx)
            raw[s, 1] = np.sum(ldy)
        elif k == "biprism":
            raw[s, 0] = np.sum(ldx * np.sign(r.x))
        elif k in ("scanner", "descanner"):
            raw[s] = [np.sum(lx), np.sum(ly), np.sum(ldx), np.sum(ldy)]
        elif k == "rotator":
            a = np.deg2rad(step["angle"])
            ca, sa = np.cos(a), np.sin(a)
            xo, yo = r.x * ca - r.y * sa, r.x * sa + r.y * ca
            dxo, dyo = r.dx * ca - r.dy * sa, r.dx * sa + r.dy * ca
            raw[s, 0] = np.sum(-lx * yo + ly * xo - ldx * dyo + ldy * dxo)
            lx, ly = lx * ca + ly * sa, -lx * sa + ly * ca
            ldx, ldy = ldx * ca + ldy * sa, -ldx * sa + ldy * ca
        elif k in ("plane", "detector", "scangrid", "source", "aperture"):
            pass
        else:
            raise NotImplementedError(k)
    return loss, raw, out


def param_grads(model, raw):
    """Per component: d loss / d (z, focal_length, def_x, def_y) from the
    per-step sums (a component's z moves the distance before it up and the
    one after it down)."""
    out = []
    n = len(model)
    for i, c in enumerate(model):
        g = {"z": raw[2 * i, 0] - (raw[2 * i + 2, 0] if i + 1 < n else 0.0)}
        if c["kind"] in ("lens", "thicklens"):
            g["focal_length"] = raw[2 * i + 1, 0]
        if c["kind"] in ("deflector", "biprism"):
            g["def_x"] = raw[2 * i + 1, 0]
        if c["kind"] == "deflector":
            g["def_y"] = raw[2 * i + 1, 1]
        out.append(g)
    return out


def margins(model, x, y, dx, dy, z=0.0):
    """Per ray, the smallest relative distance of a discrete decision from
    its threshold: |x| / max|x| at each biprism and |rr - r^2| / r^2 at each
    aperture (inf when the chain has neither)."""
    r = ORay(*(np.asarray(v, np.float64) for v in (x, y, dx, dy)), z=np.asarray(z, np.float64),
             pathlength=np.asarray(0.0))
    m = np.full(np.shape(r.x), np.inf)
    for c in model:
        r = propagate(r, comp_z(c) - r.z)
        if c["kind"] == "biprism":
            sc = np.max(np.abs(r.x)) if r.x.size else 1.0
            m = np.minimum(m, np.abs(r.x) / (sc if sc > 0 else 1.0))
        elif c["kind"] == "aperture":
            cx, cy = c.get("centre", (0.0, 0.0))
            rr = (r.x - cx) ** 2 + (r.y - cy) ** 2
            m = np.minimum(m, np.abs(rr - c["radius"] ** 2) / c["radius"] ** 2)
        r = apply_component(c, r)
    return m


def loss_complex(model, x, y, dx, dy, tx, ty, z=0.0):
    """The loss with complex arithmetic throughout (for complex-step
    derivatives of a complex-perturbed model parameter)."""
    r0 = ORay(*(np.asarray(v, np.complex128) for v in (x, y, dx, dy)), z=np.asarray(z, np.complex128),
              pathlength=np.asarray(0.0 + 0j))
    _, out = forward_tape(r0, model)
    alive = np.ones(np.shape(out.x), bool) if out.alive is None else out.alive
    rx = np.where(alive, out.x - np.asarray(tx, np.float64), 0.0)
    ry = np.where(alive, out.y - np.asarray(ty, np.float64), 0.0)
    return np.sum(rx * rx + ry * ry)


def complex_step_grads(model, x, y, dx, dy, tx, ty, h=1e-30):
    """d loss / d (z, focal_length, def_x, def_y) per component by complex step."""
    out = []
    for i, c in enumerate(model):
        g = {}
        keys = ["z"] + [k for k in ("focal_length", "def_x", "def_y") if k in c]
        for k in keys:
            m2 = [dict(cc) for cc in model]
            m2[i][k] = m2[i][k] + 1j * h
            g[k] = float(np.imag(loss_complex(m2, x, y, dx, dy, tx, ty)) / h)
        out.append(g)
    return out

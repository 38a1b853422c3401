"""Which calibration parameters the 4D-STEM fit can recover (CPU only): the
float64 oracle's Jacobian of every detector position with respect to the 21
parameters has rank 6, and the six combinations of
temgymcore_gb300.fit.identifiable_combinations span its row space: moving the
parameters along any direction that leaves the six unchanged leaves every
detector position unchanged."""
import numpy as np

import oracle
from oracle.rays import ORay


def _det(w, th):
    from temgymcore_gb300.workloads import stem_fit_probe_spec
    sg, spec = stem_fit_probe_spec(w, th, 0)
    rows, cols = w["rows"], w["cols"]
    yy, xx = np.meshgrid(np.arange(rows), np.arange(cols), indexing="ij")
    spx, spy = oracle.pixels_to_metres(sg, yy.ravel(), xx.ravel())
    dt = th.dtype
    r0 = ORay(*(w[k].astype(dt) for k in ("x", "y", "dx", "dy")), np.asarray(0.0, dt), np.asarray(0.0, dt))
    out = []
    for p in range(rows * cols):
        sp = [dict(c) for c in spec]
        for c in sp:
            if c["kind"] in ("scanner", "descanner"):
                c["scan_pos_x"], c["scan_pos_y"] = spx[p], spy[p]
        o = oracle.run_to_end(r0, sp)
        out += [o.x, o.y]
    return np.concatenate(out)


def test_fit_has_six_identifiable_combinations():
    from temgymcore_gb300.fit import identifiable_combinations
    from temgymcore_gb300.workloads import stem_fit
    w = stem_fit(seed=0, scan=(4, 5), rays_per_probe=64)
    th0 = w["theta0"]
    sc = np.abs(th0)
    sc[sc < 1e-2] = 1e-3  # the descan off-diagonals: an absolute scale
    J = np.empty((2 * 20 * 64, 21))
    for j in range(21):  # complex step: exact derivatives of the oracle
        t = th0.astype(np.complex128)
        t[j] += 1e-30j
        J[:, j] = np.imag(_det(w, t)) / 1e-30 * sc[j]
    s = np.linalg.svd(J, compute_uv=False)
    assert s[5] > 1e-7 * s[0] and np.all(s[6:] <= 1e-12 * s[0]), s / s[0]
    # the six combinations: rank 6, and their null space is the oracle's
    Jid = np.empty((6, 21))
    for j in range(21):
        h = 1e-6 * sc[j]
        tp, tm = th0.copy(), th0.copy()
        tp[j] += h
        tm[j] -= h
        Jid[:, j] = (identifiable_combinations(tp, w["gap"], 4, 5) -
                     identifiable_combinations(tm, w["gap"], 4, 5)) / (2 * h) * sc[j]
    Jid /= np.abs(Jid).max(axis=1, keepdims=True)
    u, si, vt = np.linalg.svd(Jid)
    assert si[5] > 1e-8 * si[0]
    null = vt[6:].T  # 21 x 15
    assert np.linalg.norm(J @ null) <= 1e-6 * np.linalg.norm(J)

"""The oracle's reverse-mode value-and-gradient (the checker of the batched
adjoint, and the CPU baseline's arithmetic) against complex-step derivatives
of the oracle's own forward chain, on the batched-sweep model mix (lens,
deflector, biprism, aperture) and on chains with scanners, descanners and
rotators.  CPU only."""
import numpy as np

from oracle.adjoint import complex_step_grads, margins, param_grads, value_and_raw
from oracle.rays import ORay, run_to_end


def _rays(rng, n):
    x = rng.uniform(-1e-3, 1e-3, n)
    y = rng.uniform(-1e-3, 1e-3, n)
    dx = rng.normal(0, 1e-3, n)
    dy = rng.normal(0, 1e-3, n)
    return x, y, dx, dy, rng.normal(0, 1e-3, n), rng.normal(0, 1e-3, n)


def _check(model, rays, rtol=1e-9):
    x, y, dx, dy, tx, ty = rays
    loss, raw, out = value_and_raw(model, x, y, dx, dy, tx, ty)
    ref = run_to_end(ORay(x, y, dx, dy, 0.0, 0.0), model)
    alive = np.ones(x.size, bool) if ref.alive is None else ref.alive
    assert np.isclose(loss, np.sum(((ref.x - tx) ** 2 + (ref.y - ty) ** 2)[alive]), rtol=1e-13)
    got = param_grads(model, raw)
    cs = complex_step_grads(model, x, y, dx, dy, tx, ty)
    scale = max(abs(v) for g in cs for v in g.values())
    for g, c in zip(got, cs):
        for k, v in c.items():
            assert abs(g[k] - v) <= rtol * scale, (k, g[k], v)


def test_value_and_raw_on_sweep_models():
    from temgymcore_gb300.workloads import batched_sweep
    w = batched_sweep(seed=5, n_models=12, rays=(50, 400))
    rng = np.random.default_rng(0)
    for spec in w["specs"]:
        _check(spec, _rays(rng, 300))


def test_value_and_raw_with_shifts_and_rotator():
    rng = np.random.default_rng(1)
    model = [{"kind": "scanner", "z": 0.01, "scan_pos_x": 2e-4, "scan_pos_y": -1e-4},
             {"kind": "lens", "z": 0.1, "focal_length": 0.07},
             {"kind": "rotator", "z": 0.15, "angle": 23.0},
             {"kind": "descanner", "z": 0.2, "scan_pos_x": 2e-4, "scan_pos_y": -1e-4,
              "descan_error": {"pxo_pxi": 1.01, "pyo_pyi": 0.99, "offsxi": 1e-5}},
             {"kind": "biprism", "z": 0.3, "def_x": 2e-3},
             {"kind": "aperture", "z": 0.4, "radius": 3e-3},
             {"kind": "detector", "z": 0.5, "pixel_size": (1e-5, 1e-5), "shape": (8, 8)}]
    _check(model, _rays(rng, 500))
    # the per-step sums of the scanner are d loss / d (shift)
    x, y, dx, dy, tx, ty = _rays(rng, 200)
    _, raw, _ = value_and_raw(model, x, y, dx, dy, tx, ty)
    h = 1e-30
    m2 = [dict(c) for c in model]
    m2[0]["scan_pos_x"] = m2[0]["scan_pos_x"] + 1j * h
    from oracle.adjoint import loss_complex
    cs = np.imag(loss_complex(m2, x, y, dx, dy, tx, ty)) / h
    assert np.isclose(raw[1, 0], cs, rtol=1e-9)


def test_margins_flag_decisions_near_threshold():
    model = [{"kind": "biprism", "z": 0.0, "def_x": 1e-3},
             {"kind": "aperture", "z": 0.0, "radius": 1e-3}]
    x = np.array([1e-3, 1e-9, -5e-4, 9.9999999e-4])
    y = np.zeros(4)
    m = margins(model, x, y, np.zeros(4), np.zeros(4))
    assert m[1] < 1e-5 and m[3] < 1e-6 and m[0] == 0.0 and m[2] > 0.1

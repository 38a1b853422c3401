"""Generate tests/golden/kats.json: the reference's known-answer tests as data.

The reference package (temgym_core) imports JAX, which is not installable
here, so it cannot be run to produce fixtures.  Its known answers live in its
README and test sources; this script records them (each block cites the
reference file:line it transcribes) and evaluates the closed forms those
tests compare against (analytic ABCD products built the way
tests/transfer_matrices.py builds them, with sympy; the free-space Gaussian
closed form of tests/test_gaussians.py:229-273).  Random inputs that the
reference draws unseeded are drawn here from a seeded generator.

Run:  python tests/golden/make_golden.py   (writes kats.json beside itself)
"""
from __future__ import annotations

import json
import os

import numpy as np
import sympy as sp


def prop5(z):
    """tests/transfer_matrices.py:110-143 (propagation_matrix_5x5)."""
    return sp.Matrix([[1, 0, z, 0, 0], [0, 1, 0, z, 0], [0, 0, 1, 0, 0],
                      [0, 0, 0, 1, 0], [0, 0, 0, 0, 1]])


def lens5(f):
    """tests/transfer_matrices.py:155-188 (lens_matrix_5x5)."""
    return sp.Matrix([[1, 0, 0, 0, 0], [0, 1, 0, 0, 0], [-1 / f, 0, 1, 0, 0],
                      [0, -1 / f, 0, 1, 0], [0, 0, 0, 0, 1]])


def biprism5(d):
    """tests/transfer_matrices.py:204-232 (biprism_matrix_5x5)."""
    return sp.Matrix([[1, 0, 0, 0, 0], [0, 1, 0, 0, 0], [0, 0, 1, 0, d],
                      [0, 0, 0, 1, 0], [0, 0, 0, 0, 1]])


def tolist(m):
    return [[float(v) for v in row] for row in np.array(m, dtype=np.float64)]


def main():
    rng = np.random.default_rng(20240601)
    out = {}

    # README.md:35-53 quick start; exact pathlength worked by hand = 0.88875
    out["readme_quickstart"] = {
        "source": "README.md:35-53",
        "ray": {"x": 0.1, "y": 0.2, "dx": 0.3, "dy": 0.4, "z": 0.0, "pathlength": 0.0},
        "model": [{"kind": "lens", "z": 0.5, "focal_length": 1.0},
                  {"kind": "detector", "z": 1.0, "pixel_size": [0.01, 0.01], "shape": [128, 128]}],
        "expected": {"x": 0.275, "y": 0.4, "dx": 0.05, "dy": 0.0, "z": 1.0, "pathlength": 0.88875},
        "printed_pathlength": 0.89,
    }
    # README.md:224-234 (whole-model ABCD) and README.md:240-267 (per step)
    out["readme_abcd"] = {
        "source": "README.md:224-267",
        "abcd": [[0.5, 0, 0.75, 0, 0], [0, 0.5, 0, 0.75, 0], [-1, 0, 0.5, 0, 0],
                 [0, -1, 0, 0.5, 0], [0, 0, 0, 0, 1]],
        "per_step": [tolist(prop5(0.5)), tolist(lens5(1.0)), tolist(prop5(0.5)),
                     tolist(sp.eye(5))],
    }
    # README.md:113-160 gradients: d x_out / d(f, z_lens) = (0.125, 0.1);
    # d dx_out / d x_in = -1; d dy_out / d x_in = 0
    out["readme_grads"] = {
        "source": "README.md:113-160",
        "dx_out_d_f_and_z": [0.125, 0.1],
        "ddx_out_dx_in": -1.0,
        "ddy_out_dx_in": 0.0,
    }
    # tests/test_component.py:73-101 ScanGrid metres->pixels (11x11, 0.1 m)
    out["scangrid_m2p"] = {
        "source": "tests/test_component.py:73-101",
        "grid": {"pixel_size": [0.1, 0.1], "shape": [11, 11]},
        "cases": [[[0.0, 0.0], 0.0, [5, 5]], [[-0.5, 0.5], 0.0, [0, 0]],
                  [[0.5, -0.5], 0.0, [10, 10]], [[0.0, 0.5], 0.0, [0, 5]],
                  [[-0.5, 0.0], 0.0, [5, 0]], [[0.0, 0.0], 90.0, [5, 5]],
                  [[-0.5, 0.5], 90.0, [10, 0]], [[0.5, -0.5], 90.0, [0, 10]],
                  [[0.0, 0.5], 90.0, [5, 0]], [[-0.5, 0.0], 90.0, [10, 5]]],
    }
    # tests/test_component.py:104-128 ScanGrid pixels->metres
    out["scangrid_p2m"] = {
        "source": "tests/test_component.py:104-128",
        "cases": [[[5, 5], 0.0, [0.0, 0.0]], [[0, 0], 0.0, [-0.5, 0.5]],
                  [[10, 10], 0.0, [0.5, -0.5]], [[0, 5], 0.0, [0.0, 0.5]],
                  [[5, 0], 0.0, [-0.5, 0.0]], [[5, 5], 90.0, [0.0, 0.0]],
                  [[10, 0], 90.0, [-0.5, 0.5]], [[0, 10], 90.0, [0.5, -0.5]],
                  [[5, 0], 90.0, [0.0, 0.5]], [[10, 5], 90.0, [-0.5, 0.0]]],
    }
    # tests/test_component.py:131-174 Detector both directions (no rotation)
    out["detector_m2p"] = {
        "source": "tests/test_component.py:131-150",
        "cases": [[[0.0, 0.0], [5, 5]], [[-0.5, 0.5], [0, 0]], [[0.5, -0.5], [10, 10]],
                  [[0.0, 0.5], [0, 5]], [[-0.5, 0.0], [5, 0]]],
    }
    out["detector_p2m"] = {
        "source": "tests/test_component.py:153-174",
        "cases": [[[5, 5], [0.0, 0.0]], [[0, 0], [-0.5, 0.5]], [[10, 10], [0.5, -0.5]],
                  [[0, 5], [0.0, 0.5]], [[5, 0], [-0.5, 0.0]]],
    }
    # tests/test_component.py:38-70 scan-grid symmetry shapes
    out["scangrid_symmetry_shapes"] = [[5, 5], [3, 7], [4, 4], [5, 8]]

    # tests/test_component.py:186-211 Scanner formula on random inputs
    sc = []
    for _ in range(4):
        spx, spy = rng.uniform(-5, 5, 2)
        stx, sty = rng.uniform(-0.5, 0.5, 2)
        x, y, dx, dy, z, pl = rng.uniform(-5, 5, 6)
        sc.append({"scanner": [spx, spy, stx, sty], "ray": [x, y, dx, dy, z, pl],
                   "expected": [x + spx, y + spy, dx + stx, dy + sty]})
    out["scanner"] = {"source": "tests/test_component.py:186-211", "cases": sc}

    # tests/test_component.py:214-259 Descanner formula on random inputs
    names = ["pxo_pxi", "pxo_pyi", "pyo_pxi", "pyo_pyi", "sxo_pxi", "sxo_pyi",
             "syo_pxi", "syo_pyi", "offpxi", "offpyi", "offsxi", "offsyi"]
    dc = []
    for _ in range(4):
        spx, spy = rng.uniform(-5, 5, 2)
        stx, sty = rng.uniform(-0.5, 0.5, 2)
        x, y, dx, dy, z, pl = rng.uniform(-5, 5, 6)
        e = rng.random(12)
        ex = [x + spx * e[0] + spy * e[1] + e[8] - spx,
              y + spx * e[2] + spy * e[3] + e[9] - spy,
              dx + spx * e[4] + spy * e[5] + e[10] - stx,
              dy + spx * e[6] + spy * e[7] + e[11] - sty]
        dc.append({"scan": [spx, spy, stx, sty], "err": dict(zip(names, e.tolist())),
                   "ray": [x, y, dx, dy, z, pl], "expected": ex})
    out["descanner"] = {"source": "tests/test_component.py:214-259", "cases": dc}

    # tests/test_component.py:313-353 Descanner Jacobian (5th column K1..K4)
    e = rng.random(12)
    spx, spy = 1.5, -2.0
    k = [spx * e[0] + spy * e[1] + e[8] - spx, spx * e[2] + spy * e[3] + e[9] - spy,
         spx * e[4] + spy * e[5] + e[10], spx * e[6] + spy * e[7] + e[11]]
    t = np.eye(5)
    t[0:4, 4] = k
    out["descanner_jacobian"] = {"source": "tests/test_component.py:313-353",
                                 "scan": [spx, spy], "err": dict(zip(names, e.tolist())),
                                 "expected": tolist(t)}

    # tests/test_component.py:398-407 biprism alone; :410-423 with propagation
    out["biprism"] = {"source": "tests/test_component.py:398-423",
                      "deflection": 1e-3, "z_det": 0.234,
                      "jac_dx_one": 1e-3, "prop_x_one": 1e-3 * 0.234, "prop_dx_one": 1e-3}

    # tests/test_component.py:426-465 lens + biprism chain vs analytic product
    M1, F1, defocus, defl = -10, 0.0002, 1e-4, 1e-4
    z1_l = F1 * (1 / M1 - 1)
    z2_l = F1 * (1 - M1)
    beam_z = 0.0 + defocus
    lens_z = abs(z1_l)
    bip_z = abs(z1_l) + abs(z2_l) / 2
    det_z = abs(z1_l) + abs(z2_l)
    ana = prop5(det_z - bip_z) * biprism5(defl) * prop5(bip_z - lens_z) * lens5(F1) * \
        prop5(lens_z - beam_z)
    out["lens_biprism_chain"] = {
        "source": "tests/test_component.py:426-465",
        "central_ray": {"x": -1e-15, "y": 0.0, "dx": 0.0, "dy": 0.0, "z": beam_z},
        "model": [{"kind": "source", "z": beam_z},
                  {"kind": "lens", "z": lens_z, "focal_length": F1},
                  {"kind": "biprism", "z": bip_z, "def_x": defl},
                  {"kind": "detector", "z": det_z, "pixel_size": [0.01, 0.01], "shape": [128, 128]}],
        "abcd": tolist(ana), "atol": 1e-12,
    }

    # tests/test_rays.py:15-39 paraxial propagation, :82-103 its Jacobian
    pc = []
    for _ in range(5):
        d = rng.uniform(0.1, 10.0)
        x0, y0, dx0, dy0, z0, pl0 = rng.uniform(-10, 10, 6)
        pc.append({"d": d, "ray": [x0, y0, dx0, dy0, z0, pl0],
                   "expected": [x0 + dx0 * d, y0 + dy0 * d, dx0, dy0, z0 + d, pl0 + d]})
    out["propagation"] = {"source": "tests/test_rays.py:15-39,82-103", "cases": pc}

    # tests/test_run.py:10-47 run_iter through no-op components
    out["run_iter"] = {
        "source": "tests/test_run.py:10-92",
        "ray": [0.12, 0.23, 0.34, 0.45, 3.14, 0.34],
        "model": [{"kind": "source", "z": 0.0},
                  {"kind": "scanner", "z": 1.2, "scan_pos_x": 0.0, "scan_pos_y": 0.0},
                  {"kind": "plane", "z": 1.2},
                  {"kind": "descanner", "z": 1.2, "scan_pos_x": 0.0, "scan_pos_y": 0.0},
                  {"kind": "plane", "z": 3.1}],
        "noprop_model": [{"kind": "source", "z": 1.2},
                         {"kind": "scanner", "z": 1.2, "scan_pos_x": 23.0, "scan_pos_y": 42.0},
                         {"kind": "plane", "z": 1.2},
                         {"kind": "descanner", "z": 1.2, "scan_pos_x": 13.0, "scan_pos_y": 11.0},
                         {"kind": "plane", "z": 1.2}],
        "noprop_ray": [0.12, 0.23, 0.34, 0.45, 1.2, 0.34],
    }
    # tests/test_transfer.py:137-153 accumulate order
    out["accumulate"] = {"source": "tests/test_transfer.py:137-153", "scales": [1.0, 2.0, 3.0]}

    # tests/test_gaussians.py:218-226 Qinv_ABCD identity; :229-273 free space closed form
    w0, wl, L = 1e-3, 500e-9, 0.25
    kk = 2 * np.pi / wl
    q = 1j * wl / (np.pi * w0 * w0)
    q1 = np.array([[q, 0.0], [0.0, q]], dtype=np.complex128)
    a, b = np.eye(2), L * np.eye(2)
    q2 = np.linalg.solve(a + b @ q1, np.zeros((2, 2)) + np.eye(2) @ q1)
    pref = 1.0 / np.sqrt(np.linalg.det(a + b @ q1))
    xs = np.array([-1e-4, 0.0, 2e-4])
    ys = np.array([0.0, 1e-4, -2e-4])
    r2 = np.stack(np.meshgrid(xs, ys, indexing="xy"), axis=-1).reshape(-1, 2)
    quad = np.einsum("ni,ij,nj->n", r2, q2, r2)
    field = pref * np.exp(1j * (kk / 2.0) * quad)
    out["gauss_free_space"] = {
        "source": "tests/test_gaussians.py:229-273",
        "w0": w0, "wavelength": wl, "L": L, "r2": r2.tolist(),
        "field_re": field.real.tolist(), "field_im": field.imag.tolist(), "rtol": 1e-9, "atol": 1e-12,
    }
    out["gauss_q_inv"] = {"source": "tests/test_gaussians.py:167-203",
                          "w0": 1e-3, "wavelength": 500e-9,
                          "focus_q_inv_im": 500e-9 / (np.pi * 1e-6)}
    # tests/test_gaussians.py:684-729 quadrant of a tilted beam after 1 m
    out["gauss_quadrant"] = {"source": "tests/test_gaussians.py:684-729", "z": 1.0,
                             "pixel_size": [1e-4, 1e-4], "shape": [256, 256],
                             "tilt": 1e-3, "wavelength": 500e-9, "w0": 1e-4}

    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "kats.json")
    with open(path, "w") as fh:
        json.dump(out, fh, indent=1)
    print("wrote", path)


if __name__ == "__main__":
    main()

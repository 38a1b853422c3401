"""Host-side checks (no GPU): transfer-matrix accumulation against the
reference tests (tests/test_transfer.py:152-170) and the oracle's
restatement of transfer.py:140-183 (whose loop multiplies from the last
matrix backwards); the float64 host ABCD with the direction-cosine
propagator against the oracle's complex-step Jacobian; the oracle's
direction-cosine step against the closed form of tests/test_rays.py:59-79."""
import math

import numpy as np

from oracle import transfer as OT


def test_accumulate_matrices_reference_cases():
    import temgymcore_gb300 as t
    A, B, C3 = np.eye(5), np.eye(5) * 2, np.eye(5) * 3
    for M in (A, B, C3):
        M[4, :] = [0, 0, 0, 0, 1]
    mats = [A, B, C3]
    np.testing.assert_allclose(t.accumulate_matrices(mats), C3 @ B @ A)
    np.testing.assert_allclose(t.accumulate_matrices(mats[2:3]), C3)


def test_cumulative_order_matches_oracle():
    import temgymcore_gb300 as t
    rng = np.random.default_rng(0)
    mats = rng.normal(size=(6, 5, 5))
    got = t.accumulate_matrices_cumulative(mats)
    ref = OT.accumulate_matrices_cumulative(mats)
    np.testing.assert_allclose(got, ref, rtol=1e-13, atol=1e-13)
    # the reference's order: cumulative[1] = M[-2] @ M[-1]
    np.testing.assert_allclose(got[1], mats[-2] @ mats[-1], rtol=1e-13)


def test_oracle_dircos_closed_form():
    from oracle.rays import ORay, propagate_dircos
    x0, y0, dx0, dy0, z0, pl0 = 1.0, -1.0, 2.0, 3.0, 0.5, 10.0
    d = 3.7
    r = propagate_dircos(ORay(np.array([x0]), np.array([y0]), np.array([dx0]), np.array([dy0]),
                              np.array([z0]), np.array([pl0])), d)
    n = math.sqrt(1.0 + dx0 ** 2 + dy0 ** 2)
    assert abs(r.x[0] - (x0 + (dx0 / n) / n * d)) < 1e-12
    assert abs(r.y[0] - (y0 + (dy0 / n) / n * d)) < 1e-12
    assert abs(r.z[0] - (z0 + d)) < 1e-12
    assert abs(r.pathlength[0] - (pl0 + d * n)) < 1e-12
    assert r.dx[0] == dx0 and r.dy[0] == dy0


def test_host_abcd_with_dircos_propagator():
    import oracle
    import temgymcore_gb300 as T
    from oracle.rays import ORay
    from temgymcore_gb300.workloads import build_model
    spec = [{"kind": "lens", "z": 0.1, "focal_length": 0.05},
            {"kind": "deflector", "z": 0.15, "def_x": 1e-2, "def_y": -2e-2},
            {"kind": "rotator", "z": 0.3, "angle": 37.0},
            {"kind": "detector", "z": 1.0, "pixel_size": (1e-5, 1e-5), "shape": (64, 64)}]
    for cen in ((1e-3, -2e-3, 0.2, 0.1, 0.0), (0.0, 0.0, 0.0, 0.0, 0.0), (5e-3, 1e-3, -0.3, 0.4, 0.0)):
        ref = oracle.model_abcd(ORay(*cen[:4], z=cen[4], pathlength=0.0), spec, "dircos")
        got = T.abcd_matrix(T.Ray(*cen, pathlength=0.0), build_model(spec), T.FreeSpaceDirCosine())
        np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-14)
        steps = oracle.solve_model(ORay(*cen[:4], z=cen[4], pathlength=0.0), spec, "dircos")
        got_s = T.solve_model(T.Ray(*cen, pathlength=0.0), build_model(spec), T.FreeSpaceDirCosine())
        np.testing.assert_allclose(got_s, steps, rtol=1e-12, atol=1e-14)

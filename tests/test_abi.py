"""C-ABI library: loads, exports every declared symbol, host-side ABCD (CPU only)."""
import ctypes
import glob
import os
import re

import numpy as np

from conftest import ROOT


def _declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(tg_[a-z0-9_]+)\s*\(", src))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    from temgymcore_gb300 import _native as N
    lib = N.lib()
    names = _declared()
    assert len(names) >= 8
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_status_strings_and_version():
    from temgymcore_gb300 import _native as N
    lib = N.lib()
    assert b"sm_103a" in lib.tg_version()
    assert lib.tg_status_string(0) == b"ok"
    assert lib.tg_status_string(-6) == b"workspace too small"


def test_abcd_compose_matches_golden(kats):
    import temgymcore_gb300 as T
    from temgymcore_gb300.workloads import build_model
    q = kats["readme_quickstart"]
    r = T.Ray(**q["ray"])
    model = build_model(q["model"])
    np.testing.assert_allclose(T.abcd_matrix(r, model), kats["readme_abcd"]["abcd"], atol=1e-15)
    np.testing.assert_allclose(T.solve_model(r, model), kats["readme_abcd"]["per_step"], atol=1e-15)
    c = kats["lens_biprism_chain"]
    cr = c["central_ray"]
    ray = T.Ray(x=cr["x"], y=cr["y"], dx=cr["dx"], dy=cr["dy"], z=cr["z"], pathlength=0.0)
    np.testing.assert_allclose(T.abcd_matrix(ray, build_model(c["model"])), c["abcd"], atol=c["atol"])


def test_abcd_compose_vs_oracle_random_chain():
    import oracle
    import temgymcore_gb300 as T
    from oracle.rays import ORay
    from temgymcore_gb300.workloads import build_model
    rng = np.random.default_rng(7)
    err = {k: float(v) for k, v in zip(
        ["pxo_pxi", "pxo_pyi", "pyo_pxi", "pyo_pyi", "sxo_pxi", "sxo_pyi", "syo_pxi", "syo_pyi",
         "offpxi", "offpyi", "offsxi", "offsyi"], rng.normal(0, 0.1, 12))}
    spec = [{"kind": "lens", "z": 0.1, "focal_length": 0.05},
            {"kind": "deflector", "z": 0.15, "def_x": 1e-3, "def_y": -2e-3},
            {"kind": "scanner", "z": 0.2, "scan_pos_x": 1e-6, "scan_pos_y": -2e-6, "scan_tilt_x": 1e-4},
            {"kind": "descanner", "z": 0.2, "scan_pos_x": 1e-6, "scan_pos_y": -2e-6, "descan_error": err},
            {"kind": "rotator", "z": 0.3, "angle": 37.0},
            {"kind": "biprism", "z": 0.4, "def_x": 1e-4},
            {"kind": "thicklens", "z_po": 0.5, "z_pi": 0.52, "focal_length": 0.3},
            {"kind": "aperture", "z": 0.6, "radius": 1e-2},
            {"kind": "detector", "z": 1.0, "pixel_size": (1e-5, 1e-5), "shape": (64, 64)}]
    cen = (1e-4, -2e-4, 3e-4, 1e-4, 0.0)
    ref = oracle.model_abcd(ORay(*cen[:4], z=cen[4], pathlength=0.0), spec)
    got = T.abcd_matrix(T.Ray(*cen, pathlength=0.0), build_model(spec))
    np.testing.assert_allclose(got, ref, rtol=1e-13, atol=1e-15)
    steps = oracle.solve_model(ORay(*cen[:4], z=cen[4], pathlength=0.0), spec)
    np.testing.assert_allclose(T.solve_model(T.Ray(*cen, pathlength=0.0), build_model(spec)), steps,
                               rtol=1e-13, atol=1e-15)


def test_invalid_arguments_rejected_without_gpu():
    from temgymcore_gb300 import _native as N
    lib = N.lib()
    assert lib.tg_abcd_compose(None, None, None, None) == -1
    out = (ctypes.c_double * 25)()
    cen = (ctypes.c_double * 5)()
    m = N.TgModel()
    m.n_components = 99
    assert lib.tg_abcd_compose(ctypes.byref(m), cen, out, None) == -1
    comp = (N.TgComponent * 1)()
    comp[0].kind = 42
    m.n_components = 1
    m.components = ctypes.cast(comp, ctypes.POINTER(N.TgComponent))
    assert lib.tg_abcd_compose(ctypes.byref(m), cen, out, None) == -2


def test_noalloc_size_limit_matches_its_stated_formula():
    """tg_field_direct_noalloc's size check follows the header's formula
    part(n) + 8 h w <= 32 MiB: at the largest image it passes the size check
    (the call then stops on the missing beam arrays, or without a GPU on the
    device lookup) and one row more is rejected with TG_ERR_TOO_LARGE; the
    stated capacities (about 3.2 million pixels at 32768 beams, 4.2 million
    with a few) are no larger than the formula gives."""
    import ctypes as C

    from temgymcore_gb300 import _native as N
    from temgymcore_gb300 import gaussian as G
    lib = N.lib()
    lib.tg_field_direct_noalloc.restype = C.c_int
    lib.tg_field_direct_noalloc.argtypes = [C.POINTER(N.TgModel), C.POINTER(G.TgBeams),
                                            C.POINTER(G.TgPixelMap), C.c_void_p, C.c_void_p]
    r = lambda v: (v + 255) // 256 * 256  # noqa: E731
    part = lambda n: r(r(r(96 * n) + 128 * n) + 256)  # noqa: E731
    cap = lambda n: ((32 << 20) - part(n)) // 8  # noqa: E731
    assert cap(32768) >= 3.2e6 and cap(1) >= 4.19e6
    m = N.TgModel()
    m.n_components = 0
    for n, wd in ((32768, 1000), (1, 2048), (7, 1800)):
        b = G.TgBeams()
        b.n = n  # beam arrays left NULL: nothing runs past the size check
        pm = G.TgPixelMap()
        pm.w = wd
        pm.h = cap(n) // wd
        assert lib.tg_field_direct_noalloc(C.byref(m), C.byref(b), C.byref(pm), 8, None) != -5
        pm.h += 1
        assert lib.tg_field_direct_noalloc(C.byref(m), C.byref(b), C.byref(pm), 8, None) == -5

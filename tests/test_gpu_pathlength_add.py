"""The pathlength rounding of the trace kernels (float64 base + float32 part
with float32 / integer operations) is bit-identical to the float64 add,
including binade edges, rounding ties, and every special value."""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _run(b, p):
    from temgymcore_gb300 import _native as N
    lib = N.lib()
    f = lib.tg_selftest_add_f64_f32
    f.restype = C.c_int
    f.argtypes = [C.c_void_p] * 4 + [C.c_int64, C.c_void_p]
    bt = torch.tensor(b, dtype=torch.float64, device="cuda")
    pt = torch.tensor(p, dtype=torch.float32, device="cuda")
    fast, ref = torch.empty_like(bt), torch.empty_like(bt)
    N.check(f(bt.data_ptr(), pt.data_ptr(), fast.data_ptr(), ref.data_ptr(), bt.numel(), N.stream_ptr()),
            "tg_selftest_add_f64_f32")
    fast, ref = fast.cpu().numpy(), ref.cpu().numpy()
    # the float64 add on the device is the float64 add on the host
    np.testing.assert_array_equal(ref.view(np.int64)[~np.isnan(ref)],
                                  (np.asarray(b) + np.asarray(p, np.float32).astype(np.float64))
                                  .view(np.int64)[~np.isnan(ref)])
    return fast, ref


def _same_bits(fast, ref):
    nan = np.isnan(ref)
    assert np.array_equal(np.isnan(fast), nan)
    bad = np.nonzero(fast.view(np.int64)[~nan] != ref.view(np.int64)[~nan])[0]
    assert bad.size == 0, bad[:10]


def test_add_f64_f32_random_and_edges(cuda):
    rng = np.random.default_rng(11)
    n = 1 << 20
    # metre-scale bases with micrometre-scale float32 parts (the trace case)
    b1 = rng.choice([-1.0, 1.0], n) * rng.uniform(0.1, 4.0, n)
    p1 = rng.normal(0, 1e-6, n).astype(np.float32)
    # every exponent in and around the fast range, p from far below to above ulp(b) * 2^22
    eb = rng.uniform(-90, 200, n)
    b2 = rng.choice([-1.0, 1.0], n) * np.exp2(eb) * rng.uniform(1, 2, n)
    with np.errstate(over="ignore"):  # float32 overflow to inf is one of the cases
        p2 = (rng.choice([-1.0, 1.0], n) * np.abs(b2) * np.exp2(rng.uniform(-70, 2, n))).astype(np.float32)
    # binade edges: b on or just beside a power of two, p pushing across it
    pw = np.exp2(rng.integers(-60, 150, n).astype(np.float64))
    up = np.nextafter(pw, np.inf)
    dn = np.nextafter(pw, 0)
    b3 = np.choose(rng.integers(0, 3, n), [up, dn, pw]) * rng.choice([-1.0, 1.0], n)
    ulp = np.spacing(np.abs(b3))
    p3 = (rng.integers(-6, 7, n) * 0.5 * ulp * rng.choice([1.0, 0.999, 1.001, 2.0], n)).astype(np.float32)
    # exact ties with odd and even significands
    b4 = 1.0 + rng.integers(0, 1 << 20, n) * 2.0 ** -52
    p4 = (rng.choice([-1.0, 1.0], n) * rng.choice([0.5, 1.5, 2.5, 3.5], n) * 2.0 ** -52).astype(np.float32)
    specials_b = np.array([0.0, -0.0, 5e-324, -5e-324, 2.2250738585072014e-308, np.inf, -np.inf, np.nan,
                           1.0, -1.0, 2.0 ** -75, 2.0 ** -76, 2.0 ** 178, 2.0 ** 179, 1.7976931348623157e308])
    specials_p = np.array([0.0, -0.0, 1e-45, -1e-45, 1.17549435e-38, np.inf, -np.inf, np.nan,
                           1.0, -1.0, 3.4028235e38, 1e-7, -1e-7, 2.0 ** -53, -2.0 ** -54], np.float32)
    b5 = np.repeat(specials_b, specials_p.size)
    p5 = np.tile(specials_p, specials_b.size)
    b = np.concatenate([b1, b2, b3, b4, b5])
    p = np.concatenate([p1, p2, p3, p4, p5]).astype(np.float32)
    fast, ref = _run(b, p)
    _same_bits(fast, ref)

"""Host side of the ray sources (no GPU): the ring count the C ABI reports
for a requested number of rays equals the reference's concentric_rings
count (utils.py:117-175, restated in the oracle)."""
import ctypes as C

from oracle import sources as OS


def test_ring_counts_match_reference():
    from temgymcore_gb300 import _native as N
    import temgymcore_gb300.sources  # noqa: F401  (registers the entry points)
    for num in (1, 2, 3, 5, 7, 10, 31, 100, 999, 1000, 4096, 12345, 54321, 100000):
        n = C.c_int64(0)
        assert N.lib().tg_source_count(num, 0, C.byref(n)) == 0
        assert n.value == OS.concentric_rings(num, 1.0).shape[0], num
    n = C.c_int64(0)
    assert N.lib().tg_source_count(777, 1, C.byref(n)) == 0 and n.value == 777
    assert N.lib().tg_source_count(0, 0, C.byref(n)) == -1

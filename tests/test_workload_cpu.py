"""The host-side workload generators behind the mixed-size benchmark: the
class trace is deterministic per seed and uniform over the nine classes, so
its mean request size is the figure the roofline's algorithmic bytes use
(2 x E[size] per malloc/free pair)."""
from __future__ import annotations

import numpy as np

from gallatin_gb300.workload import class_bytes, mixed_class_trace, mixed_mean_bytes


def test_mixed_trace_is_deterministic_and_round_major():
    a = mixed_class_trace(1 << 12, 3, 42)
    b = mixed_class_trace(1 << 12, 3, 42)
    assert a.shape == (3, 1 << 12) and a.dtype == np.uint8
    assert np.array_equal(a, b)
    assert not np.array_equal(a, mixed_class_trace(1 << 12, 3, 43))
    assert not np.array_equal(a[0], a[1])  # each round draws again
    assert int(a.max()) <= 8


def test_mixed_trace_is_uniform_over_the_classes():
    n = 1 << 20
    trace = mixed_class_trace(n, 2, 42).reshape(-1)
    counts = np.bincount(trace, minlength=9)
    expected = trace.size / 9
    assert np.all(np.abs(counts - expected) < 0.01 * expected), counts
    mean = float((np.uint64(16) << trace.astype(np.uint64)).mean())
    assert abs(mean - mixed_mean_bytes()) < 0.005 * mixed_mean_bytes()


def test_mean_bytes_is_the_roofline_figure():
    assert mixed_mean_bytes() == 8176 / 9
    assert round(2 * mixed_mean_bytes(), 1) == 1816.9


def test_class_bytes_rounds_up_to_a_power_of_two_of_at_least_16():
    sizes = np.array([1, 15, 16, 17, 1000, 1024, 1025, 4096, 4097, (1 << 40) + 1], dtype=np.uint64)
    want = np.array([16, 16, 16, 32, 1024, 1024, 2048, 4096, 8192, 1 << 41], dtype=np.uint64)
    assert np.array_equal(class_bytes(sizes), want)

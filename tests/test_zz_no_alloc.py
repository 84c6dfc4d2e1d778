"""The allocation-free host entry point, for callers that may not allocate
device memory while they run: a serving loop that cannot take the
device-wide synchronisation of cudaMalloc, or a process whose device memory
was divided among pools up front. It keeps its scratch in a fixed array
inside the library. Collected last on purpose: if it fails, a run that stops
at the first failure has already run every other test."""
from __future__ import annotations

import numpy as np
import pytest

import gallatin_gb300 as gal

pytestmark = pytest.mark.gpu


def test_noalloc_entry_point_matches_allocating_one(cuda):
    from gallatin_gb300.workload import mixed_class_trace

    n, rounds, seed = 1 << 17, 8, 42  # a 1 MiB trace, inside the 2 MiB scratch
    trace = mixed_class_trace(n, rounds, seed).reshape(-1).copy()
    host = cuda.from_numpy(trace).pin_memory()
    kw = dict(seg_every=64, seg_lo=16 << 20, seg_hi=64 << 20)
    # the allocating entry point on one handle, the allocation-free one on a
    # fresh handle of its own, so it cannot borrow the other's scratch
    with gal.Gallatin.generate_on_device(1 << 30, seed, print_info=False) as a, \
            gal.Gallatin.generate_on_device(1 << 30, seed, print_info=False) as b:
        want = a.run_mixed_host(n, rounds, seed, host.data_ptr(), **kw)
        first = b.run_mixed_host_noalloc(n, rounds, seed, host.data_ptr(), **kw)
        cuda.cuda.synchronize()
        # after the first call (which may load the array's module) the device's
        # free memory must not move, call after call
        free_before, _ = cuda.cuda.mem_get_info()
        second = b.run_mixed_host_noalloc(n, rounds, seed, host.data_ptr(), **kw)
        third = b.run_mixed_host_noalloc(n, rounds, seed, host.data_ptr(), **kw)
        cuda.cuda.synchronize()
        free_after, _ = cuda.cuda.mem_get_info()
        assert want[0] == 0 and want[1] == 0, want
        assert np.array_equal(first, want), (first, want)
        assert np.array_equal(second, want), (second, want)  # stats restart from zero
        assert np.array_equal(third, want), (third, want)
        assert int(want[2] + want[3]) == n // 256 // 64
        assert free_after == free_before, f"device free memory moved by {free_before - free_after} bytes"


def test_noalloc_rejects_traces_beyond_its_scratch(cuda):
    with gal.Gallatin.generate_on_device(256 << 20, 1, print_info=False) as a:
        big = np.zeros(gal.NOALLOC_TRACE_MAX_BYTES + 1, dtype=np.uint8)
        with pytest.raises(gal.GalError, match="static scratch"):
            a.run_mixed_host_noalloc(len(big), 1, 1, big.ctypes.data)

"""The glibc replays behind the CPU baselines of the spill and calloc
workloads run the same traces as the device kernels and see no failures."""
from __future__ import annotations

import numpy as np

import oracle
from gallatin_gb300.workload import mixed_class_trace


def test_fill_drain_replay_verifies_every_allocation():
    classes = mixed_class_trace(50_000, 1, 42).reshape(-1)
    secs, misses, bad = oracle.cpu_replay_fill_drain(classes, workers=3)
    assert secs > 0 and misses == 0 and bad == 0


def test_zeroed_replay_sees_only_zeroed_allocations():
    secs, misses, bad = oracle.cpu_replay_mixed_zeroed(20_000, 0, 20_000, 3, 42, workers=2)
    assert secs > 0 and misses == 0 and bad == 0


def test_zeroed_replay_reads_the_same_class_trace():
    trace = mixed_class_trace(4096, 2, 7)
    a = oracle.cpu_replay_mixed_zeroed(4096, 0, 4096, 2, 7, workers=1, classes=np.ascontiguousarray(trace))
    assert a[1] == 0 and a[2] == 0

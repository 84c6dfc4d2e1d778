"""Synthetic request traces for the benchmark workloads (host side, numpy).

mixed_class_trace reproduces on the host the size sequence the mixed
workload kernel draws on the device: per thread an xorshift64 stream seeded
with splitmix64(seed + tid), class = x mod 9, size = 16 << class. The trace
is what the host-buffer entry point (gal_run_mixed_host) copies to the GPU.
"""
from __future__ import annotations

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64(x: np.ndarray) -> np.ndarray:
    x = x.astype(np.uint64) + np.uint64(0x9E3779B97F4A7C15)
    x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return x ^ (x >> np.uint64(31))


def mixed_class_trace(n_threads: int, rounds: int, seed: int) -> np.ndarray:
    """uint8 classes, shape (rounds, n_threads), round-major like the device reads it."""
    with np.errstate(over="ignore"):
        s = splitmix64(np.arange(n_threads, dtype=np.uint64) + np.uint64(seed))
        out = np.empty((rounds, n_threads), dtype=np.uint8)
        for r in range(rounds):
            s ^= (s << np.uint64(13)) & _M64
            s ^= s >> np.uint64(7)
            s ^= (s << np.uint64(17)) & _M64
            out[r] = (s % np.uint64(9)).astype(np.uint8)
    return out


def mixed_mean_bytes() -> float:
    """Mean request size of the mixed workload: the mean of 16 << k, k = 0..8."""
    return sum(16 << k for k in range(9)) / 9.0

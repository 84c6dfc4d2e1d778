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


def class_bytes(sizes: np.ndarray) -> np.ndarray:
    """Power-of-two size class of each request, at least 16 B."""
    s = np.maximum(sizes.astype(np.uint64), np.uint64(16))
    e = np.ceil(np.log2(s.astype(np.float64))).astype(np.int64)
    e += (np.uint64(1) << e.astype(np.uint64)) < s  # float rounding guard
    return np.uint64(1) << e.astype(np.uint64)


def batch_trace(
    seed: int = 42,
    n_batches: int = 64,
    batch_lo: int = 1024,
    batch_hi: int = 524288,
    mu: float = float(np.log(256.0)),
    sigma: float = 1.5,
    size_lo: int = 16,
    size_hi: int = 64 << 20,
    p_malloc: float = 0.6,
    drain: bool = True,
):
    """Request stream of the batching configuration.

    n_batches batches with sizes uniform in [batch_lo, batch_hi]; each request
    is a malloc (probability p_malloc) of a lognormal(mu, sigma) size clipped
    to [size_lo, size_hi], or a free of a slot chosen uniformly from the
    allocations live at the start of the batch. Requests are u64
    (slot << 32 | size; size 0 = free), shuffled within a batch. With `drain`
    a last batch frees everything still live, so a launch starts and ends
    with an empty live set.

    info["peak_class_bytes"] bounds the bytes the live set holds at any point
    when each request is rounded up to its power-of-two size class (the live
    set before a batch plus every malloc of the batch).

    Returns (requests u64[], offsets u64[batches + 1], table_slots, info)."""
    rng = np.random.default_rng(seed)
    slot_bytes = np.zeros(0, dtype=np.uint64)
    live_bytes = 0
    peak_bytes = 0
    counts = rng.integers(batch_lo, batch_hi + 1, size=n_batches)
    live = np.empty(0, dtype=np.uint64)
    recycled = np.empty(0, dtype=np.uint64)
    next_slot = 0
    chunks, offsets = [], [0]
    mallocs = frees = 0
    max_size = 0
    max_live = 0
    for n in counts:
        n = int(n)
        n_free = min(int(rng.binomial(n, 1.0 - p_malloc)), len(live))
        n_malloc = n - n_free
        if n_free:
            pick = rng.choice(len(live), size=n_free, replace=False)
            keep = np.ones(len(live), dtype=bool)
            keep[pick] = False
            freed = live[pick]
            live = live[keep]
        else:
            freed = np.empty(0, dtype=np.uint64)
        reuse = min(n_malloc, len(recycled))
        fresh = n_malloc - reuse
        slots = np.concatenate([recycled[len(recycled) - reuse :], np.arange(next_slot, next_slot + fresh, dtype=np.uint64)])
        recycled = recycled[: len(recycled) - reuse]
        next_slot += fresh
        sizes = np.clip(np.rint(rng.lognormal(mu, sigma, size=n_malloc)), size_lo, size_hi).astype(np.uint64)
        if n_malloc:
            max_size = max(max_size, int(sizes.max()))
        if next_slot > len(slot_bytes):
            slot_bytes = np.concatenate([slot_bytes, np.zeros(next_slot - len(slot_bytes), dtype=np.uint64)])
        cls = class_bytes(sizes)
        freed_bytes = int(slot_bytes[freed].sum()) if n_free else 0
        peak_bytes = max(peak_bytes, live_bytes + int(cls.sum()))
        live_bytes += int(cls.sum()) - freed_bytes
        slot_bytes[freed] = 0
        slot_bytes[slots] = cls
        batch = np.concatenate([(slots << np.uint64(32)) | sizes, freed << np.uint64(32)])
        rng.shuffle(batch)
        chunks.append(batch)
        offsets.append(offsets[-1] + n)
        recycled = np.concatenate([recycled, freed])
        live = np.concatenate([live, slots])
        mallocs += n_malloc
        frees += n_free
        max_live = max(max_live, len(live))
    if drain and len(live):
        chunks.append(live << np.uint64(32))
        offsets.append(offsets[-1] + len(live))
        frees += len(live)
    reqs = np.concatenate(chunks).astype(np.uint64)
    info = {
        "batches": len(offsets) - 1,
        "requests": int(len(reqs)),
        "mallocs": mallocs,
        "frees": frees,
        "max_live": max_live,
        "max_request_bytes": max_size,
        "peak_class_bytes": peak_bytes,
    }
    return reqs, np.array(offsets, dtype=np.uint64), next_slot, info


def prefix_with_drain(reqs: np.ndarray, offsets: np.ndarray, k: int):
    """The first k batches of a request stream, then one batch that frees every
    slot those batches leave live, so the prefix also starts and ends with an
    empty live set. Returns (requests, offsets)."""
    k = min(k, len(offsets) - 1)
    head = np.asarray(reqs[: int(offsets[k])], dtype=np.uint64)
    slots = head >> np.uint64(32)
    is_malloc = (head & np.uint64(0xFFFFFFFF)) != 0
    # the last request naming a slot decides whether it is live
    rev_slots = slots[::-1]
    uniq, first_in_rev = np.unique(rev_slots, return_index=True)
    live = uniq[is_malloc[::-1][first_in_rev]]
    out = np.concatenate([head, live.astype(np.uint64) << np.uint64(32)])
    offs = np.concatenate([np.asarray(offsets[: k + 1], dtype=np.uint64), [np.uint64(len(out))]])
    return out, offs.astype(np.uint64)

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


# ---- serving ---------------------------------------------------------------

def serving_trace(
    seed: int = 42,
    steps: int = 600,
    arrivals_per_step: float = 1000.0,
    median_tokens: float = 1024.0,
    sigma: float = 1.0,
    min_tokens: int = 128,
    max_tokens: int = 32768,
    tokens_per_page: int = 16,
):
    """Streams of the serving configuration.

    Arrivals are Poisson: arrivals_per_step = rate x simulated step length
    (2,000 streams/s x 0.5 s per 16-token step = 1,000). Stream lengths are
    lognormal(ln median, sigma) tokens clipped to [min, max]; a stream needs
    ceil(tokens / tokens_per_page) pages and takes one per step.

    Returns a dict of numpy arrays: arrival_step (u32, ascending), tokens
    (u32), pages (u32), page_prefix (u64, n+1: pages of streams before i),
    arrivals_end (u32, steps+1: arrivals_end[s + 1] streams arrived at steps
    <= s), plus steps and tokens_per_page."""
    rng = np.random.default_rng(seed)
    per_step = rng.poisson(arrivals_per_step, size=steps)
    n = int(per_step.sum())
    arrival_step = np.repeat(np.arange(steps, dtype=np.uint32), per_step)
    tokens = np.clip(np.rint(rng.lognormal(np.log(median_tokens), sigma, size=n)), min_tokens, max_tokens).astype(np.uint32)
    pages = ((tokens + tokens_per_page - 1) // tokens_per_page).astype(np.uint32)
    page_prefix = np.zeros(n + 1, dtype=np.uint64)
    np.cumsum(pages, out=page_prefix[1:])
    arrivals_end = np.zeros(steps + 1, dtype=np.uint32)
    np.cumsum(per_step, out=arrivals_end[1:])
    return {"arrival_step": arrival_step, "tokens": tokens, "pages": pages, "page_prefix": page_prefix,
            "arrivals_end": arrivals_end, "steps": steps, "tokens_per_page": tokens_per_page}


def single_stream(trace: dict, i: int, extra_steps: int = 2) -> dict:
    """A trace holding only stream i of `trace`, arriving at step 0, with its
    original id (so its tokens, and its checksum, are the ones it has in the
    full trace)."""
    p = int(trace["pages"][i])
    steps = p + extra_steps
    arrivals_end = np.ones(steps + 1, dtype=np.uint32)
    arrivals_end[0] = 0
    return {"arrival_step": np.zeros(1, dtype=np.uint32), "tokens": trace["tokens"][i:i + 1].copy(),
            "pages": trace["pages"][i:i + 1].copy(), "page_prefix": np.array([0, p], dtype=np.uint64),
            "arrivals_end": arrivals_end, "steps": steps, "tokens_per_page": trace["tokens_per_page"],
            "ids": np.array([i], dtype=np.uint32)}


def serving_admission(trace: dict, budget_pages: int, max_slots: int, slot_delay: int = 1):
    """Host model of the serving loop's first-come-first-served admission (the
    device loop must reproduce it exactly). At step s, k_s streams are
    admitted: the largest k such that they have arrived by step s, k free slots
    exist, and the pages committed to admitted, unfinished streams plus their
    pages stay within budget_pages. Every admitted stream takes one page per
    step; a stream with p pages admitted at step a finishes at step a + p - 1;
    its pages count as free for the admission of step a + p and its slot, which
    the loop reuses only after the stream's pages are freed in step a + p, for
    step a + p + slot_delay.

    Returns (admit_step u32[n], 0xFFFFFFFF = never admitted within the steps;
    per-step arrays: admitted, committed pages after the step's admissions)."""
    steps = trace["steps"]
    pages = trace["pages"].astype(np.int64)
    prefix = trace["page_prefix"]
    arrivals_end = trace["arrivals_end"]
    n = len(pages)
    admit = np.full(n, 0xFFFFFFFF, dtype=np.uint32)
    release_pages = np.zeros(steps + 2, dtype=np.int64)
    release_slots = np.zeros(steps + 2, dtype=np.int64)
    nxt = 0
    committed = 0
    free_slots = max_slots
    out_k = np.zeros(steps, dtype=np.int64)
    out_committed = np.zeros(steps, dtype=np.int64)
    for s in range(steps):
        committed -= release_pages[s]
        free_slots += release_slots[s]
        hi = min(int(arrivals_end[s + 1]), nxt + free_slots)
        room = budget_pages - committed
        lim = int(prefix[nxt]) + room
        k = int(np.searchsorted(prefix[nxt:hi + 1], lim, side="right")) - 1 if hi > nxt else 0
        k = max(k, 0)
        if k:
            admit[nxt:nxt + k] = s
            p = pages[nxt:nxt + k]
            committed += int(p.sum())
            free_slots -= k
            fin = s + p
            np.add.at(release_pages, np.minimum(fin, steps + 1), p)
            np.add.at(release_slots, np.minimum(fin + slot_delay, steps + 1), 1)
            nxt += k
        out_k[s] = k
        out_committed[s] = committed
    return admit, {"admitted": out_k, "committed": out_committed}


# ---- data structures ---------------------------------------------------------

def vector_lengths(n: int = 1_000_000, median: float = 64.0, sigma: float = 1.5, cap: int = 65536,
                   seed: int = 42) -> np.ndarray:
    """Target lengths of the per-thread vectors: lognormal(ln median, sigma)
    rounded, clipped to [1, cap] (u32)."""
    rng = np.random.default_rng(seed)
    return np.clip(np.rint(rng.lognormal(np.log(median), sigma, size=n)), 1, cap).astype(np.uint32)

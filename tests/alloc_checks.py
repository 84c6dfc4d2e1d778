"""Invariant checks on allocator output and metadata snapshots (test helpers).

The invariants come from the workload definitions the allocator is judged on:
no overlapping live allocations, alignment to min(size class, segment), the
right size class for every pointer (via the memory table), and, after every
allocation is freed and the pinned blocks are flushed, trees and tables equal
to their initial state.
"""
from __future__ import annotations

import numpy as np

import gallatin_gb300 as gal


def class_bytes(alloc: gal.Gallatin, size: int) -> int:
    tier, tree, cnt = gal.classify(size, alloc.min_size, alloc.max_size, alloc.segment_size)
    if tier == "segment":
        return cnt * alloc.segment_size
    if tier == "block":
        return alloc.min_size * 4096 << tree
    return (alloc.min_size << tree) * cnt


def spans_of(alloc: gal.Gallatin, ptrs: np.ndarray, sizes: np.ndarray):
    live = ptrs != 0
    out = []
    for p, s in zip(ptrs[live], sizes[live]):
        out.append((int(p), int(p) + class_bytes(alloc, int(s)), int(s)))
    return out


def check_no_overlap(spans) -> None:
    spans = sorted(spans)
    for (s0, e0, z0), (s1, e1, z1) in zip(spans, spans[1:]):
        assert e0 <= s1, f"overlap: [{s0:#x},{e0:#x}) size {z0} and [{s1:#x},{e1:#x}) size {z1}"


def check_alignment_and_bounds(alloc: gal.Gallatin, spans) -> None:
    base, end = alloc.arena_base, alloc.arena_base + alloc.arena_bytes
    for s, e, size in spans:
        assert base <= s and e <= end, f"allocation outside the arena: {s:#x}"
        align = min(class_bytes(alloc, size), alloc.segment_size)
        assert (s - base) % align == 0, f"size {size} at offset {s - base:#x} not aligned to {align}"


def _block_state(alloc: gal.Gallatin, off: int, tree: int) -> str:
    """The meta word fields of the block holding arena offset `off` (for failure messages)."""
    seg_shift = alloc.segment_size.bit_length() - 1
    block_shift = alloc.min_size.bit_length() - 1 + 12
    b = ((off >> seg_shift) << (seg_shift - block_shift)) + ((off & (alloc.segment_size - 1)) >> (block_shift + tree))
    m = int(alloc.dump("block_meta")[b])
    counters = {k: v for k, v in alloc.stats()["counters"].items() if v}
    return (f"block {b}: live {m & 0xFFFFFFFF} tree {(m >> 32) & 0xFF} state {(m >> 40) & 3} run {(m >> 42) & 15} "
            f"flags {(m >> 46) & 3} cursor {m >> 48}; counters {counters}")


def check_size_classes(alloc: gal.Gallatin, spans) -> None:
    ids = alloc.dump("chunk_ids")
    seg_shift = alloc.segment_size.bit_length() - 1
    for s, _, size in spans:
        seg = (s - alloc.arena_base) >> seg_shift
        tier, tree, cnt = gal.classify(size, alloc.min_size, alloc.max_size, alloc.segment_size)
        want = alloc.num_trees + 1 + cnt if tier == "segment" else tree
        if int(ids[seg]) != want:
            bad = sum(1 for s2, _, z2 in spans if int(ids[(s2 - alloc.arena_base) >> seg_shift]) == gal.GAL_FREE_SEGMENT)
            detail = _block_state(alloc, s - alloc.arena_base, tree) if tier == "slice" else ""
            raise AssertionError(f"size {size} at offset {s - alloc.arena_base:#x}: segment {seg} tagged "
                                 f"{int(ids[seg])}, want {want} ({bad} allocations in untagged segments; "
                                 f"tags {ids.tolist()[:48]}); {detail}")


def check_live(alloc, ptrs, sizes) -> list:
    spans = spans_of(alloc, ptrs, sizes)
    check_no_overlap(spans)
    check_alignment_and_bounds(alloc, spans)
    check_size_classes(alloc, spans)
    return spans


def full_layers(universe: int) -> list[np.ndarray]:
    import oracle

    shape = oracle.veb_shape(universe)
    out, u = [], universe
    for words in reversed(shape):
        layer = np.zeros(words, dtype=np.uint64)
        for w in range(words):
            left = u - 64 * w
            layer[w] = np.uint64(0xFFFFFFFFFFFFFFFF) if left >= 64 else np.uint64((1 << left) - 1)
        out.append(layer)
        u = (u - 1) // 64 + 1
    return list(reversed(out))


def check_restored(alloc: gal.Gallatin) -> None:
    """After all frees and flush_pinned: the initial state, bit for bit."""
    seg_layers = alloc.veb_layers(-1)
    for got, want in zip(seg_layers, full_layers(alloc.num_segments)):
        assert np.array_equal(got, want), "segment tree not restored"
    for t in range(alloc.num_trees):
        for layer in alloc.veb_layers(t):
            assert not layer.any(), f"sub tree {t} not empty"
    for k in range(alloc.num_classes):
        for kind in ("adopt_tree", "roomy_tree"):
            for layer in alloc.veb_layers(k, kind):
                assert not layer.any(), f"{kind} of slot class {k} not empty"
    ids = alloc.dump("chunk_ids")
    assert (ids == gal.GAL_FREE_SEGMENT).all(), "memory table not reset"
    avail = alloc.dump("seg_avail")
    assert (avail == gal.GAL_SEG_GATE).all(), "segment gates not reset"
    meta = alloc.dump("block_meta")
    state = (meta >> np.uint64(40)) & np.uint64(3)
    live = meta & np.uint64(0xFFFFFFFF)
    assert (state == 0).all(), "blocks left outside their pools"
    assert (live == 0).all(), "live counts not balanced"
    slots = alloc.dump("slots")
    assert (slots == gal.GAL_EMPTY_BLOCK).all()
    assert int(alloc.dump("locks")[0]) == 0
    c = alloc.stats()["counters"]
    assert c["corrupt"] == 0 and c["bad_free"] == 0, c

"""Host-arena allocators, device-first allocation with a host fallback, and
zeroed (calloc) allocation.

Follows the reference's host and fused paths (generate_on_device_host,
gallatin.cuh:423-526; global_malloc_fused / global_free_fused,
global_allocator.cuh:186-216; test shape tests/src/global_exceed_test.cu:
38-110) and its running_calloc mode (gallatin.cuh:1306-1369). The checks are
the allocator invariants: no overlap, alignment and size class in whichever
arena served a pointer, every write read back, both allocators restored
after the drain, and, for calloc, every byte of every allocation zero when
handed out.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import gallatin_gb300 as gal
from alloc_checks import check_live, check_restored

pytestmark = pytest.mark.gpu

STAT_MISS, STAT_BAD, STAT_HOST = 0, 1, 4


def fill_sizes(n: int, seed: int) -> np.ndarray:
    """16 << class_i from a class trace the test owns (the kernels' d_classes)."""
    rng = np.random.default_rng(seed)
    return rng.integers(0, 9, size=n, dtype=np.uint8)


def run_fill_drain(cuda, dev, host, classes, check_filled=None):
    """Fill, then check_filled(ptrs) on the live set the fill left, then drain."""
    n = len(classes)
    d_classes = cuda.from_numpy(classes).cuda()
    d_table = cuda.zeros(n, dtype=cuda.int64, device="cuda")
    d_stats = cuda.zeros(8, dtype=cuda.int64, device="cuda")
    dev.run_fused(host, n, 0, d_table.data_ptr(), d_stats.data_ptr(), d_classes=d_classes.data_ptr(), phases=1)
    cuda.cuda.synchronize()
    ptrs = d_table.cpu().numpy().view(np.uint64).copy()
    fill_stats = d_stats.cpu().numpy().copy()
    if check_filled is not None:
        check_filled(ptrs)
    dev.run_fused(host, n, 0, d_table.data_ptr(), d_stats.data_ptr(), d_classes=d_classes.data_ptr(), phases=2)
    cuda.cuda.synchronize()
    return ptrs, fill_stats, d_stats.cpu().numpy(), d_table.cpu().numpy()


@pytest.mark.parametrize("rep", range(4))
def test_fused_spills_to_the_host_arena_and_restores_both(cuda, rep):
    # 4 device segments cannot hold 131,072 mixed allocations (~113 MiB):
    # the rest must land in the host arena, and every pointer must verify
    dev = gal.Gallatin.generate_on_device(64 << 20, 3 + rep, print_info=False)
    host = gal.Gallatin.generate_on_device_host(512 << 20, 4 + rep, print_info=False)
    try:
        assert host.host_arena and not dev.host_arena
        classes = fill_sizes(1 << 17, 11 + rep)
        sizes = (np.uint64(16) << classes.astype(np.uint64))
        where = {}

        def check_filled(ptrs):
            # invariants per arena, on the live set the fill phase left
            on_dev = (ptrs >= dev.arena_base) & (ptrs < dev.arena_base + dev.arena_bytes)
            on_host = (ptrs >= host.arena_base) & (ptrs < host.arena_base + host.arena_bytes)
            assert (on_dev ^ on_host).all(), "every pointer is in exactly one arena"
            check_live(dev, np.where(on_dev, ptrs, 0), sizes)
            check_live(host, np.where(on_host, ptrs, 0), sizes)
            where["host"] = int(on_host.sum())

        ptrs, fill_stats, drain_stats, table = run_fill_drain(cuda, dev, host, classes, check_filled)
        assert fill_stats[STAT_MISS] == 0
        assert int(fill_stats[STAT_HOST]) == where["host"]
        assert 0 < where["host"] < len(ptrs)
        assert drain_stats[STAT_BAD] == 0
        assert not table.any(), "drain clears the table"
        for a in (dev, host):
            a.flush_pinned()
            cuda.cuda.synchronize()
            check_restored(a)
    finally:
        dev.free_on_device()
        host.free_on_device()


def test_fused_without_host_arena_returns_null_when_full(cuda):
    dev = gal.Gallatin.generate_on_device(64 << 20, 5, print_info=False)
    try:
        classes = fill_sizes(1 << 17, 12)
        sizes = (np.uint64(16) << classes.astype(np.uint64))
        ptrs, fill_stats, drain_stats, _ = run_fill_drain(cuda, dev, None, classes,
                                                          lambda p: check_live(dev, p, sizes))
        misses = int(fill_stats[STAT_MISS])
        assert misses > 0 and misses == int((ptrs == 0).sum())
        assert fill_stats[STAT_HOST] == 0 and drain_stats[STAT_BAD] == 0
        dev.flush_pinned()
        cuda.cuda.synchronize()
        check_restored(dev)
    finally:
        dev.free_on_device()


def test_host_arena_bytes_are_visible_to_the_cpu(cuda):
    # the fill writes i and ~i into each allocation from the GPU; the CPU reads
    # them back at the same addresses (pinned, mapped host memory)
    # 32 segments: every size class gets segments of its own
    host = gal.Gallatin.generate_on_device_host(512 << 20, 6, print_info=False)
    try:
        classes = fill_sizes(4096, 13)
        n = len(classes)
        d_classes = cuda.from_numpy(classes).cuda()
        d_table = cuda.zeros(n, dtype=cuda.int64, device="cuda")
        d_stats = cuda.zeros(8, dtype=cuda.int64, device="cuda")
        host.run_fused(None, n, 0, d_table.data_ptr(), d_stats.data_ptr(), d_classes=d_classes.data_ptr(), phases=1)
        cuda.cuda.synchronize()
        ptrs = d_table.cpu().numpy().view(np.uint64)
        assert (ptrs != 0).all()
        # the CPU dereferences these addresses: every allocation must lie
        # inside the host arena first, so a bad pointer fails the test
        # instead of faulting the process
        sizes = np.uint64(16) << classes.astype(np.uint64)
        lo, hi = host.arena_base, host.arena_base + host.arena_bytes
        inside = (ptrs >= np.uint64(lo)) & (ptrs + sizes <= np.uint64(hi))
        assert inside.all(), f"{int((~inside).sum())} allocations outside the host arena"
        for i in range(0, n, 97):
            size = 16 << int(classes[i])
            first = ctypes.c_uint64.from_address(int(ptrs[i])).value
            last = ctypes.c_uint64.from_address(int(ptrs[i]) + size - 8).value
            assert first == i and last == (~i) & 0xFFFFFFFFFFFFFFFF
        host.run_fused(None, n, 0, d_table.data_ptr(), d_stats.data_ptr(), d_classes=d_classes.data_ptr(), phases=2)
        cuda.cuda.synchronize()
        assert int(d_stats[STAT_BAD]) == 0
        host.flush_pinned()
        cuda.cuda.synchronize()
        check_restored(host)
    finally:
        host.free_on_device()


def test_fused_host_entry_point_matches_device_run(cuda):
    dev = gal.Gallatin.generate_on_device(64 << 20, 7, print_info=False)
    host = gal.Gallatin.generate_on_device_host(512 << 20, 8, print_info=False)
    try:
        classes = fill_sizes(1 << 17, 14)
        for _ in range(2):
            out = dev.run_fused_host(host, len(classes), 0, classes.ctypes.data)
            assert out[STAT_MISS] == 0 and out[STAT_BAD] == 0 and 0 < out[STAT_HOST] < len(classes)
        for a in (dev, host):
            a.flush_pinned()
            cuda.cuda.synchronize()
            check_restored(a)
    finally:
        dev.free_on_device()
        host.free_on_device()


@pytest.mark.parametrize(
    "big",
    [(0, 0, 0), (8, 64 << 10, 2 << 20), (64, 20 << 20, 40 << 20)],
    ids=["slices-and-runs", "block-tier", "segment-tier"],
)
def test_calloc_allocations_read_zero(cuda, big):
    big_every, lo, hi = big
    a = gal.Gallatin.generate_on_device(1 << 30, 21, print_info=False, running_calloc=True)
    try:
        assert a.calloc
        d_stats = cuda.zeros(8, dtype=cuda.int64, device="cuda")
        a.run_zeroed(1 << 16, 4, 5, d_stats.data_ptr(), big_every=big_every, big_lo=lo or 1, big_hi=hi or 1)
        cuda.cuda.synchronize()
        st = d_stats.cpu().numpy()
        assert st[STAT_MISS] == 0 and st[STAT_BAD] == 0, st
        a.flush_pinned()
        cuda.cuda.synchronize()
        check_restored(a)
    finally:
        a.free_on_device()


def test_calloc_check_sees_dirty_bytes_without_calloc(cuda):
    # the same workload on an allocator that does not zero: slices reused
    # after the first round still hold the previous owner's fill
    a = gal.Gallatin.generate_on_device(1 << 30, 21, print_info=False)
    try:
        d_stats = cuda.zeros(8, dtype=cuda.int64, device="cuda")
        a.run_zeroed(1 << 16, 4, 5, d_stats.data_ptr())
        cuda.cuda.synchronize()
        st = d_stats.cpu().numpy()
        assert st[STAT_MISS] == 0 and st[STAT_BAD] > 0, st
    finally:
        a.free_on_device()


def test_calloc_on_a_host_arena(cuda):
    a = gal.Gallatin.generate_on_device_host(1 << 30, 22, print_info=False, running_calloc=True)
    try:
        assert a.calloc and a.host_arena
        d_stats = cuda.zeros(8, dtype=cuda.int64, device="cuda")
        a.run_zeroed(1 << 14, 3, 6, d_stats.data_ptr(), big_every=16, big_lo=64 << 10, big_hi=1 << 20)
        cuda.cuda.synchronize()
        st = d_stats.cpu().numpy()
        assert st[STAT_MISS] == 0 and st[STAT_BAD] == 0, st
        a.flush_pinned()
        cuda.cuda.synchronize()
        check_restored(a)
    finally:
        a.free_on_device()


def test_calloc_batches_stream(cuda):
    # the batched stream frees through the same device free: with calloc on
    # it still serves every request and restores the allocator
    from gallatin_gb300 import workload

    reqs, offsets, slots, _ = workload.batch_trace(seed=3, n_batches=6, batch_lo=1024, batch_hi=65536)
    a = gal.Gallatin.generate_on_device(2 << 30, 23, print_info=False, running_calloc=True)
    try:
        out = a.run_batches_host(reqs, offsets, slots, persistent=True, binned=True)
        assert out[STAT_MISS] == 0
        a.flush_pinned()
        cuda.cuda.synchronize()
        check_restored(a)
    finally:
        a.free_on_device()


@pytest.mark.parametrize("rep", range(4))
@pytest.mark.parametrize("calloc", [False, True], ids=["plain", "calloc"])
def test_mixed_rounds_in_a_full_arena_never_share_a_slice(cuda, calloc, rep):
    # 262,144 threads x 4 rounds of malloc / fill / verify / free against 4
    # segments: most rounds find the arena full. Any slice handed to two
    # owners at once shows up as a verify failure (each fills it with its own
    # value and reads it back)
    a = gal.Gallatin.generate_on_device(64 << 20, 31, print_info=False, running_calloc=calloc)
    try:
        d_stats = cuda.zeros(8, dtype=cuda.int64, device="cuda")
        a.run_mixed(1 << 18, 4, 9 + rep, d_stats.data_ptr())
        cuda.cuda.synchronize()
        st = d_stats.cpu().numpy()
        assert st[STAT_MISS] > 0 and st[STAT_BAD] == 0, st
        a.flush_pinned()
        cuda.cuda.synchronize()
        check_restored(a)
    finally:
        a.free_on_device()

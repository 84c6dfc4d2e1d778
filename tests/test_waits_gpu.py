"""Bounded waits end with an error status the host reads, not a hang.

The reference spins without bound on its segment-tier lock
(gallatin.cuh:796) and on per-tree attach locks (gallatin.cuh:1559). Here
every wait has a limit; when it runs out the request returns NULL and the
allocator counts a timeout. The tests hold a lock from the host
(gal_set_locks writes the lock word while no kernel runs, so no thread ever
releases it), make one request wait on it, and read NULL and the counter;
then they clear the lock and see the same request succeed. Nothing faults,
traps or hangs the GPU: the waits are short by construction."""
from __future__ import annotations

import time

import numpy as np
import pytest

import gallatin_gb300 as gal
from alloc_checks import check_restored

pytestmark = pytest.mark.gpu

SEGMENT_LOCK = 1 << 31


def malloc_one(torch, alloc, size: int) -> int:
    d_sizes = torch.tensor([size], dtype=torch.int64, device="cuda")
    d_ptrs = torch.zeros(1, dtype=torch.int64, device="cuda")
    alloc.malloc_batch(d_sizes.data_ptr(), 1, d_ptrs.data_ptr())
    torch.cuda.synchronize()
    return int(d_ptrs.cpu().numpy().view(np.uint64)[0])


def free_one(torch, alloc, ptr: int) -> None:
    d_ptrs = torch.from_numpy(np.array([ptr], dtype=np.uint64).view(np.int64)).cuda()
    alloc.free_batch(d_ptrs.data_ptr(), 1)
    torch.cuda.synchronize()


def test_held_segment_lock_times_out_then_serves(cuda):
    with gal.Gallatin.generate_on_device(256 << 20, 3, print_info=False) as a:
        a.set_wait_limit(2000)  # 2000 tries, at most ~1 us each
        a.set_locks(SEGMENT_LOCK)
        t0 = time.perf_counter()
        p = malloc_one(cuda, a, 32 << 20)  # two segments: the segment tier
        waited = time.perf_counter() - t0
        c = a.stats()["counters"]
        assert p == 0, "a request behind a held lock must not be served"
        assert c["timeout"] == 1 and c["oom_segment"] == 0, c
        assert waited < 2.0, f"the bounded wait took {waited:.3f} s"
        a.set_locks(0)
        p = malloc_one(cuda, a, 32 << 20)
        assert p != 0 and a.stats()["counters"]["timeout"] == 1
        free_one(cuda, a, p)
        a.flush_pinned()
        cuda.cuda.synchronize()
        check_restored(a)


def test_held_tree_lock_times_out_a_block_request(cuda):
    # a block-tier request (64 KiB: a whole block of tree 0) finds no segment
    # formatted for its tree and must take tree 0's attach lock to format
    # one; with the lock held it gives up after its attempt budget
    with gal.Gallatin.generate_on_device(256 << 20, 4, print_info=False) as a:
        a.set_locks(1 << 0)
        p = malloc_one(cuda, a, 64 << 10)
        c = a.stats()["counters"]
        assert p == 0 and c["timeout"] == 1 and c["oom_block"] == 1, c
        a.set_locks(0)
        p = malloc_one(cuda, a, 64 << 10)
        assert p != 0
        free_one(cuda, a, p)
        a.flush_pinned()
        cuda.cuda.synchronize()
        check_restored(a)
        assert a.check_restored()["restored"]

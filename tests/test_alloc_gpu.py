"""Allocator invariants on the GPU: no overlap, alignment, size class, null only
when the arena cannot fit, and a fully restored state after everything is freed."""
from __future__ import annotations

import numpy as np
import pytest

import gallatin_gb300 as gal
from alloc_checks import check_live, check_restored, class_bytes

pytestmark = pytest.mark.gpu


def malloc_batch(torch, alloc, sizes: np.ndarray) -> np.ndarray:
    d_sizes = torch.from_numpy(sizes.astype(np.uint64).view(np.int64)).cuda()
    d_ptrs = torch.zeros(len(sizes), dtype=torch.int64, device="cuda")
    alloc.malloc_batch(d_sizes.data_ptr(), len(sizes), d_ptrs.data_ptr())
    torch.cuda.synchronize()
    return d_ptrs.cpu().numpy().view(np.uint64).copy()


def free_batch(torch, alloc, ptrs: np.ndarray) -> None:
    d_ptrs = torch.from_numpy(ptrs.astype(np.uint64).view(np.int64)).cuda()
    alloc.free_batch(d_ptrs.data_ptr(), len(ptrs))
    torch.cuda.synchronize()


def release_all(torch, alloc, ptrs) -> None:
    free_batch(torch, alloc, ptrs)
    alloc.flush_pinned()
    torch.cuda.synchronize()
    check_restored(alloc)


TIER_SIZES = [1, 16, 17, 33, 100, 256, 1000, 2048, 4096, 4097, 8192, 12000, 32768, 40000, 1 << 20, 3 << 20,
              16 << 20, (16 << 20) + 1, 50 << 20]
TIER_P = np.array([8, 8, 8, 8, 8, 8, 8, 8, 8, 4, 4, 4, 4, 2, 1, 1, 0.5, 0.3, 0.2])


def longest_free_run(alloc) -> int:
    leaf = alloc.veb_layers(-1)[-1]
    bits = np.unpackbits(leaf.view(np.uint8), bitorder="little")[: alloc.num_segments]
    longest = run = 0
    for b in bits:
        run = run + 1 if b else 0
        longest = max(longest, run)
    return longest


def check_nulls_justified(alloc, ptrs, sizes) -> None:
    """In a malloc-only phase the free space only shrinks, so every null must
    still be justified by the end state: no free run long enough for a
    segment-tier request, and no free segment at all for the other tiers."""
    failed = sizes[ptrs == 0]
    if failed.size == 0:
        return
    longest = longest_free_run(alloc)
    for s in failed:
        tier, _, cnt = gal.classify(int(s), alloc.min_size, alloc.max_size, alloc.segment_size)
        need = cnt if tier == "segment" else 1
        assert longest < need, f"request of {int(s)} B failed while {longest} contiguous segments are free"


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_mixed_tiers_batch(cuda, seed):
    rng = np.random.default_rng(seed)
    with gal.Gallatin.generate_on_device(2 << 30, seed, print_info=False) as a:
        sizes = rng.choice(TIER_SIZES, size=20000, p=TIER_P / TIER_P.sum()).astype(np.uint64)
        ptrs = malloc_batch(cuda, a, sizes)
        check_live(a, ptrs, sizes)
        check_nulls_justified(a, ptrs, sizes)
        assert (ptrs != 0).mean() > 0.5
        release_all(cuda, a, ptrs)


def test_interleaved_phases_reuse_freed_slices(cuda):
    rng = np.random.default_rng(9)
    with gal.Gallatin.generate_on_device(1 << 30, 5, print_info=False) as a:
        live_p, live_s = np.zeros(0, np.uint64), np.zeros(0, np.uint64)
        for phase in range(6):
            sizes = (16 << rng.integers(0, 9, size=30000)).astype(np.uint64)
            ptrs = malloc_batch(cuda, a, sizes)
            assert (ptrs != 0).all(), "a half-empty arena returned null"
            live_p, live_s = np.concatenate([live_p, ptrs]), np.concatenate([live_s, sizes])
            check_live(a, live_p, live_s)
            drop = rng.random(len(live_p)) < 0.6
            free_batch(cuda, a, live_p[drop])
            live_p, live_s = live_p[~drop], live_s[~drop]
        release_all(cuda, a, live_p)


def test_one_class_packs_blocks(cuda):
    with gal.Gallatin.generate_on_device(512 << 20, 42, print_info=False) as a:
        n = 1 << 20
        ptrs = malloc_batch(cuda, a, np.full(n, 16, dtype=np.uint64))
        assert (ptrs != 0).all()
        check_live(a, ptrs, np.full(n, 16, dtype=np.uint64))
        blocks = np.unique((ptrs - np.uint64(a.arena_base)) >> np.uint64(16))
        # 4096 slices per 64 KiB block; a pinned block is swapped out once it
        # holds 7/8 of that, and partly filled pinned blocks remain
        assert len(blocks) <= n // (4096 * 7 // 8) + a.slot_count[0]
        release_all(cuda, a, ptrs)


def make_arena(nbytes, seed, host):
    """A device-arena allocator, or the same over pinned host memory (the
    reference's generate_on_device_host; its tests fill it to capacity the
    same way, tests/src/gallatin_host_test.cu:136-200)."""
    make = gal.Gallatin.generate_on_device_host if host else gal.Gallatin.generate_on_device
    return make(nbytes, seed, print_info=False)


# the capacity and out-of-memory results depend on how concurrent claims
# race, so each such test runs several times per session
REPEATS = 8


@pytest.mark.parametrize("rep", range(REPEATS))
@pytest.mark.parametrize("host", [False, True], ids=["device-arena", "host-arena"])
def test_slice_tier_fills_to_capacity_then_returns_null(cuda, host, rep):
    # 4 segments of 16 MiB; a 4 KiB block is a whole segment: 4 * 4096 slices
    with make_arena(64 << 20, 3 + rep, host) as a:
        cap = 4 * 4096
        sizes = np.full(cap + 100, 4096, dtype=np.uint64)
        ptrs = malloc_batch(cuda, a, sizes)
        assert int((ptrs != 0).sum()) == cap
        check_live(a, ptrs, sizes)
        assert a.stats()["free_segments"] == 0
        release_all(cuda, a, ptrs)


@pytest.mark.parametrize("rep", range(REPEATS // 2))
@pytest.mark.parametrize("host", [False, True], ids=["device-arena", "host-arena"])
def test_block_and_segment_tiers_exact_capacity(cuda, host, rep):
    with make_arena(64 << 20, 4 + rep, host) as a:
        ptrs = malloc_batch(cuda, a, np.full(5, 16 << 20, dtype=np.uint64))  # whole-segment blocks
        assert int((ptrs != 0).sum()) == 4
        free_batch(cuda, a, ptrs)
        a.flush_pinned()
        ptrs = malloc_batch(cuda, a, np.full(3, 32 << 20, dtype=np.uint64))  # 2-segment runs
        assert int((ptrs != 0).sum()) == 2
        check_live(a, ptrs, np.full(3, 32 << 20, dtype=np.uint64))
        release_all(cuda, a, ptrs)


def test_segment_tier_fails_only_without_a_free_run(cuda):
    rng = np.random.default_rng(12)
    with gal.Gallatin.generate_on_device(48 * (16 << 20), 8, print_info=False) as a:
        sizes = (rng.integers(1, 9, size=40) * (16 << 20)).astype(np.uint64)
        ptrs = malloc_batch(cuda, a, sizes)
        check_live(a, ptrs, sizes)
        check_nulls_justified(a, ptrs, sizes)
        assert (ptrs != 0).any()
        release_all(cuda, a, ptrs)


def test_pairs_and_mixed_workloads_are_clean(cuda):
    with gal.Gallatin.generate_on_device(2 << 30, 42, print_info=False) as a:
        stats = cuda.zeros(8, dtype=cuda.int64, device="cuda")
        a.run_pairs(1 << 20, 16, stats.data_ptr(), block_dim=1024)
        a.run_mixed(1 << 18, 4, 42, stats.data_ptr(), seg_every=64, seg_lo=16 << 20, seg_hi=64 << 20)
        cuda.cuda.synchronize()
        st = stats.cpu().numpy()
        assert st[0] == 0, f"slice/block misses: {st}"
        assert st[1] == 0, f"verify failures: {st}"
        assert st[2] + st[3] == (1 << 18) // 256 // 64
        a.flush_pinned()
        cuda.cuda.synchronize()
        check_restored(a)


def test_mixed_trace_matches_generated_sizes(cuda):
    """The host-buffer entry point over a class trace equals the device-seeded run."""
    from gallatin_gb300.workload import mixed_class_trace

    n, rounds = 1 << 16, 3
    trace = mixed_class_trace(n, rounds, 42)
    import oracle

    assert np.array_equal(trace, oracle.cpu_mixed_classes(n, rounds, 42))
    with gal.Gallatin.generate_on_device(1 << 30, 42, print_info=False) as a:
        host = cuda.from_numpy(trace.reshape(-1).copy()).pin_memory()
        out = a.run_mixed_host(n, rounds, 42, host.data_ptr())
        assert out[0] == 0 and out[1] == 0


def test_global_allocator_mirror(cuda):
    a = gal.init_global_allocator(256 << 20, 111, print_info=False)
    try:
        sizes = np.array([16, 64, 4096, 9000, 70000], dtype=np.uint64)
        ptrs = malloc_batch(cuda, gal.global_allocator(), sizes)
        assert (ptrs != 0).all()
        check_live(a, ptrs, sizes)
        gal.print_global_stats()
        free_batch(cuda, a, ptrs)
    finally:
        gal.free_global_allocator()


def test_bad_free_is_counted_not_fatal(cuda):
    with gal.Gallatin.generate_on_device(64 << 20, 1, print_info=False) as a:
        bogus = np.array([a.arena_base + 12345, 8, a.arena_base + a.arena_bytes + 64], dtype=np.uint64)
        free_batch(cuda, a, bogus)
        assert a.stats()["counters"]["bad_free"] == 3
        a.reset_counters()
        assert a.stats()["counters"]["bad_free"] == 0


def test_allocated_size_spans_are_disjoint_per_class(cuda):
    with gal.Gallatin.generate_on_device(256 << 20, 2, print_info=False) as a:
        for size in (16, 4096, 8192, 40000):
            assert class_bytes(a, size) >= size


def test_restore_report_agrees_with_the_host_check(cuda):
    """gal_check_restored sees what check_restored sees: a live allocation
    (negative control), then nothing once it is freed and the slots flushed."""
    with gal.Gallatin.generate_on_device(256 << 20, 21, print_info=False) as a:
        sizes = np.array([16, 4096, 8192, 100_000, 40 << 20], dtype=np.uint64)
        ptrs = malloc_batch(cuda, a, sizes)
        assert (ptrs != 0).all()
        a.flush_pinned()
        cuda.cuda.synchronize()
        rep = a.check_restored()
        assert not rep["restored"]
        assert rep["tagged_segments"] >= 4 and rep["live_blocks"] >= 3 and rep["taken_slices"] >= 3, rep
        with pytest.raises(AssertionError):
            check_restored(a)
        release_all(cuda, a, ptrs)
        rep = a.check_restored()
        assert rep["restored"], rep


def test_mixed_full_configuration_restores_the_initial_state(cuda):
    """The mixed-size configuration at full size: an 8 GiB arena, 4,194,304
    threads x 8 rounds of malloc / fill / verify / free over 16..4096 B, plus
    256 segment-tier requests of 16-256 MiB. No NULL, no verify failure, and
    after the pinned blocks are flushed every tree and table is back in its
    initial state."""
    from gallatin_gb300.workload import mixed_class_trace

    n, rounds = 4_194_304, 8
    trace = mixed_class_trace(n, rounds, 42)
    with gal.Gallatin.generate_on_device(8 << 30, 42, print_info=False) as a:
        d_trace = cuda.from_numpy(trace.reshape(-1)).cuda()
        stats = cuda.zeros(8, dtype=cuda.int64, device="cuda")
        a.run_mixed(n, rounds, 42, stats.data_ptr(), seg_every=64, seg_lo=16 << 20, seg_hi=256 << 20,
                    d_classes=d_trace.data_ptr(), block_dim=256)
        cuda.cuda.synchronize()
        st = stats.cpu().numpy()
        assert st[0] == 0 and st[1] == 0, f"misses / verify failures: {st}"
        assert st[2] + st[3] == n // 256 // 64
        a.flush_pinned()
        cuda.cuda.synchronize()
        rep = a.check_restored()
        assert rep["restored"], rep
        check_restored(a)


@pytest.mark.parametrize("drop_freed", [False, True], ids=["lines-kept", "lines-dropped"])
def test_freed_lines_dropped_or_kept_leave_every_allocation_intact(cuda, drop_freed):
    """With drop_freed, free drops the L2 lines of freed 128 B..4 KiB slices
    (discard, no write-back); by default it leaves them. Either way every
    byte each owner writes reads back (the next owner writes after the
    discard), nothing is NULL, and the state restores."""
    with gal.Gallatin.generate_on_device(2 << 30, 13, print_info=False, drop_freed=drop_freed) as a:
        assert bool(a.flags & gal.FLAG_DROP_FREED) == drop_freed
        stats = cuda.zeros(8, dtype=cuda.int64, device="cuda")
        for rep in range(3):
            a.run_mixed(1 << 18, 6, 100 + rep, stats.data_ptr(), seg_every=64, seg_lo=16 << 20, seg_hi=64 << 20)
        a.run_pairs(1 << 20, 256, stats.data_ptr(), block_dim=1024)
        cuda.cuda.synchronize()
        st = stats.cpu().numpy()
        assert st[0] == 0 and st[1] == 0, st
        a.flush_pinned()
        cuda.cuda.synchronize()
        check_restored(a)

"""Batched request streams: the persistent kernel, its CUDA graph and the plain
per-batch path serve the same stream with the same outcome, and the allocator
ends empty."""
from __future__ import annotations

import numpy as np
import pytest

import gallatin_gb300 as gal
from alloc_checks import check_live, check_restored

pytestmark = pytest.mark.gpu


def small_trace(seed=5):
    from gallatin_gb300.workload import batch_trace

    return batch_trace(seed, n_batches=12, batch_lo=1024, batch_hi=40000)


@pytest.mark.parametrize("persistent,binned,width",
                         [(False, False, 32), (True, False, 32), (True, False, 16), (True, False, 8),
                          (True, True, 32), (True, True, 8)])
def test_batches_serve_stream_and_restore(cuda, persistent, binned, width):
    reqs, offsets, slots, info = small_trace()
    with gal.Gallatin.generate_on_device(1 << 30, 3, print_info=False) as a:
        d_reqs = cuda.from_numpy(reqs.view(np.int64)).cuda()
        d_offs = cuda.from_numpy(offsets.view(np.int64)).cuda()
        d_table = cuda.zeros(slots + 1, dtype=cuda.int64, device="cuda")
        stats = cuda.zeros(8, dtype=cuda.int64, device="cuda")
        # all but the drain batch: the table then holds the live set
        a.run_batches(d_reqs.data_ptr(), d_offs.data_ptr(), offsets[:-1], d_table.data_ptr(), stats.data_ptr(),
                      width=width, persistent=persistent, binned=binned)
        cuda.cuda.synchronize()
        assert int(stats[0]) == 0
        table = d_table.cpu().numpy().view(np.uint64)
        # sizes of the live slots, from the host replay of the stream
        sizes = np.zeros(slots + 1, dtype=np.uint64)
        for r in reqs[: int(offsets[-2])]:
            slot, size = int(r >> np.uint64(32)), int(r & np.uint64(0xFFFFFFFF))
            sizes[slot] = size
        live = table != 0
        check_live(a, table[live], sizes[live])
        # the drain batch frees the rest
        drain = offsets[-2:]
        d_drain = cuda.from_numpy((drain - drain[0]).view(np.int64)).cuda()
        d_reqs_drain = cuda.from_numpy(reqs[int(drain[0]):].view(np.int64).copy()).cuda()
        a.run_batches(d_reqs_drain.data_ptr(), d_drain.data_ptr(), drain - drain[0], d_table.data_ptr(),
                      stats.data_ptr(), width=width, persistent=persistent, binned=binned)
        a.flush_pinned()
        cuda.cuda.synchronize()
        assert not d_table.any()
        check_restored(a)


@pytest.mark.parametrize("persistent,binned", [(False, False), (True, False), (True, True)])
def test_graph_replay_repeats_the_stream(cuda, persistent, binned):
    reqs, offsets, slots, info = small_trace(7)
    with gal.Gallatin.generate_on_device(1 << 30, 4, print_info=False) as a:
        d_reqs = cuda.from_numpy(reqs.view(np.int64)).cuda()
        d_offs = cuda.from_numpy(offsets.view(np.int64)).cuda()
        d_table = cuda.zeros(slots + 1, dtype=cuda.int64, device="cuda")
        stats = cuda.zeros(8, dtype=cuda.int64, device="cuda")
        with a.capture_batches(d_reqs.data_ptr(), d_offs.data_ptr(), offsets, d_table.data_ptr(),
                               stats.data_ptr(), persistent=persistent, binned=binned) as g:
            for _ in range(3):
                g.launch()
            cuda.cuda.synchronize()
        assert int(stats[0]) == 0
        assert not d_table.any()  # every replay ends with the drain batch
        a.flush_pinned()
        cuda.cuda.synchronize()
        check_restored(a)


def test_batches_host_entry_point(cuda):
    reqs, offsets, slots, info = small_trace(9)
    with gal.Gallatin.generate_on_device(1 << 30, 4, print_info=False) as a:
        out = a.run_batches_host(reqs, offsets, slots, persistent=True)
        assert out[0] == 0
        out = a.run_batches_host(reqs, offsets, slots, persistent=False, width=16)
        assert out[0] == 0
        out = a.run_batches_host(reqs, offsets, slots, persistent=True, binned=True, ctas_per_sm=2)
        assert out[0] == 0


def test_reference_plain_path_on_the_same_stream(cuda):
    import oracle

    if oracle.load_ref() is None:
        pytest.skip("reference build not available on this box")
    reqs, offsets, slots, info = small_trace(11)
    assert info["max_request_bytes"] <= 16 << 20  # never the reference's segment tier
    ref = oracle.RefGallatin(1 << 30, 4)
    try:
        d_reqs = cuda.from_numpy(reqs.view(np.int64)).cuda()
        d_offs = cuda.from_numpy(offsets.view(np.int64)).cuda()
        d_table = cuda.zeros(slots + 1, dtype=cuda.int64, device="cuda")
        stats = cuda.zeros(8, dtype=cuda.int64, device="cuda")
        ref.run_batches(d_reqs.data_ptr(), d_offs.data_ptr(), offsets, d_table.data_ptr(), stats.data_ptr())
        cuda.cuda.synchronize()
        assert int(stats[0]) == 0
        assert not d_table.any()
    finally:
        ref.close()


@pytest.mark.parametrize("persistent,binned", [(False, False), (True, False), (True, True)])
def test_long_lived_random_frees_fit_half_full_arena(cuda, persistent, binned):
    """Allocations live across many batches and are freed in random order, the
    live set peaking at about half the arena in size-class bytes: no request
    may fail, and the state restores after the drain."""
    from gallatin_gb300.workload import batch_trace

    reqs, offsets, slots, info = batch_trace(5, n_batches=40, batch_lo=1024, batch_hi=131072)
    arena = 1280 << 20
    assert info["peak_class_bytes"] <= arena // 2
    with gal.Gallatin.generate_on_device(arena, 6, print_info=False) as a:
        d_reqs = cuda.from_numpy(reqs.view(np.int64)).cuda()
        d_offs = cuda.from_numpy(offsets.view(np.int64)).cuda()
        d_table = cuda.zeros(slots + 1, dtype=cuda.int64, device="cuda")
        stats = cuda.zeros(8, dtype=cuda.int64, device="cuda")
        a.run_batches(d_reqs.data_ptr(), d_offs.data_ptr(), offsets, d_table.data_ptr(), stats.data_ptr(),
                      persistent=persistent, binned=binned)
        cuda.cuda.synchronize()
        c = a.stats()["counters"]
        assert int(stats[0]) == 0, c
        assert c["timeout"] == 0 and c["corrupt"] == 0, c
        a.flush_pinned()
        cuda.cuda.synchronize()
        check_restored(a)


@pytest.mark.parametrize("rep", range(3))
def test_binned_path_serves_each_request_like_the_plain_path(cuda, rep):
    """Binning only reorders a batch: every malloc gets a block of its own
    size class and the live set after each form is the same set of slots."""
    reqs, offsets, slots, info = small_trace(13 + rep)
    tables = []
    for persistent, binned in [(False, False), (True, True)]:
        with gal.Gallatin.generate_on_device(1 << 30, 8, print_info=False) as a:
            d_reqs = cuda.from_numpy(reqs.view(np.int64)).cuda()
            d_offs = cuda.from_numpy(offsets.view(np.int64)).cuda()
            d_table = cuda.zeros(slots + 1, dtype=cuda.int64, device="cuda")
            stats = cuda.zeros(8, dtype=cuda.int64, device="cuda")
            a.run_batches(d_reqs.data_ptr(), d_offs.data_ptr(), offsets[:-1], d_table.data_ptr(), stats.data_ptr(),
                          persistent=persistent, binned=binned)
            cuda.cuda.synchronize()
            assert int(stats[0]) == 0
            table = d_table.cpu().numpy().view(np.uint64)
            sizes = np.zeros(slots + 1, dtype=np.uint64)
            for r in reqs[: int(offsets[-2])]:
                sizes[int(r >> np.uint64(32))] = int(r & np.uint64(0xFFFFFFFF))
            live = table != 0
            check_live(a, table[live], sizes[live])
            tables.append(live)
    assert np.array_equal(tables[0], tables[1])


@pytest.mark.parametrize("rep", range(3))
@pytest.mark.parametrize("arena_mib,calloc,binned", [(64, False, False), (128, False, True), (64, True, True)],
                         ids=["64MiB-plain", "128MiB-binned", "64MiB-calloc-binned"])
def test_batches_in_an_arena_too_small_for_the_stream(cuda, arena_mib, calloc, binned, rep):
    # the stream's live set peaks near 90 MB in class bytes, over nine slice
    # trees and the block tier: a 4- or 8-segment arena runs out. Mallocs
    # return NULL (the strike path), what was served must still be a valid
    # live set, frees of NULL slots are no-ops, and the drain restores the state
    reqs, offsets, slots, info = small_trace(11)
    with gal.Gallatin.generate_on_device(arena_mib << 20, 6 + rep, print_info=False, running_calloc=calloc) as a:
        d_reqs = cuda.from_numpy(reqs.view(np.int64)).cuda()
        d_offs = cuda.from_numpy(offsets.view(np.int64)).cuda()
        d_table = cuda.zeros(slots + 1, dtype=cuda.int64, device="cuda")
        stats = cuda.zeros(8, dtype=cuda.int64, device="cuda")
        a.run_batches(d_reqs.data_ptr(), d_offs.data_ptr(), offsets[:-1], d_table.data_ptr(), stats.data_ptr(),
                      persistent=binned, binned=binned)
        cuda.cuda.synchronize()
        assert int(stats[0]) > 0, "the arena should have run out"
        table = d_table.cpu().numpy().view(np.uint64)
        sizes = np.zeros(slots + 1, dtype=np.uint64)
        for r in reqs[: int(offsets[-2])]:
            slot, size = int(r >> np.uint64(32)), int(r & np.uint64(0xFFFFFFFF))
            sizes[slot] = size
        live = table != 0
        assert live.any()
        check_live(a, table[live], sizes[live])
        drain = offsets[-2:]
        d_drain = cuda.from_numpy((drain - drain[0]).view(np.int64)).cuda()
        d_reqs_drain = cuda.from_numpy(reqs[int(drain[0]):].view(np.int64).copy()).cuda()
        a.run_batches(d_reqs_drain.data_ptr(), d_drain.data_ptr(), drain - drain[0], d_table.data_ptr(),
                      stats.data_ptr(), persistent=binned, binned=binned)
        a.flush_pinned()
        cuda.cuda.synchronize()
        assert not d_table.any()
        check_restored(a)

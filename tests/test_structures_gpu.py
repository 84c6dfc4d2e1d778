"""Allocator-backed data structures on the GPU: the chained hash table keeps
every inserted key with its value through erase, compaction and reinsert;
the doubling vectors keep every pushed item; and the allocator ends as it
started once the structures are freed."""
from __future__ import annotations

import numpy as np
import pytest

import gallatin_gb300 as gal
from alloc_checks import check_restored
from gallatin_gb300.workload import vector_lengths

pytestmark = pytest.mark.gpu

N = 1 << 20
BUCKETS = N // 4


def zeros(cuda):
    return cuda.zeros(8, dtype=cuda.int64, device="cuda")


def read(cuda, st):
    cuda.cuda.synchronize()
    return st.cpu().numpy()


@pytest.mark.parametrize("explicit_keys", [False, True])
def test_table_lifecycle(cuda, explicit_keys):
    with gal.Gallatin.generate_on_device(2 << 30, 3, print_info=False, min_size=128) as a:
        keys = None
        if explicit_keys:
            rng = np.random.default_rng(5)
            host = rng.integers(0, 2**63, size=N, dtype=np.int64)
            keys = cuda.from_numpy(host).cuda()
        kp = keys.data_ptr() if keys is not None else None
        with a.table(BUCKETS, seed=9) as t:
            st = zeros(cuda)
            t.op("insert", N, st.data_ptr(), d_keys=kp)
            assert read(cuda, st)[0] == 0
            t.op("query", N, st.data_ptr(), d_keys=kp)
            s = read(cuda, st)
            assert s[1] == 0 and s[2] == 0
            longest, nodes = t.chain_stats()
            assert nodes >= N // 7 and longest < 16
            t.op("erase_half", N, st.data_ptr(), d_keys=kp)
            t.op("query_after_erase", N, st.data_ptr(), d_keys=kp)
            s = read(cuda, st)
            assert s[1] == 0 and s[2] == 0
            t.op("compact", 0, st.data_ptr())
            freed = int(read(cuda, st)[3])
            assert t.chain_stats()[1] == nodes - freed
            t.op("reinsert_half", N, st.data_ptr(), d_keys=kp)
            t.op("query", N, st.data_ptr(), d_keys=kp)
            s = read(cuda, st)
            assert s[0] == 0 and s[1] == 0 and s[2] == 0
            _, nodes2 = t.chain_stats()
            st2 = zeros(cuda)
            t.op("clear", 0, st2.data_ptr())
            assert read(cuda, st2)[3] == nodes2
        # nodes are 120 B: they took 128 B slices (tree 0 of a 128 B minimum)
        assert a.stats()["tree_pins"][0] > 0
        a.flush_pinned()
        cuda.cuda.synchronize()
        check_restored(a)


def test_vectors_grow_and_keep_their_items(cuda):
    lengths = vector_lengths(1 << 16, seed=3)
    assert lengths.max() > 4096  # some vectors grow into multi-slice backings
    d_len = cuda.from_numpy(lengths.view(np.int32)).cuda()
    with gal.Gallatin.generate_on_device(2 << 30, 4, print_info=False, min_size=128) as a:
        for _ in range(2):
            st = zeros(cuda)
            a.run_vectors(d_len.data_ptr(), len(lengths), st.data_ptr(), start=1)
            s = read(cuda, st)
            assert s[0] == 0 and s[2] == 0
            assert s[4] == int(lengths.sum())
        a.flush_pinned()
        cuda.cuda.synchronize()
        check_restored(a)


def test_reference_allocator_runs_the_same_structures(cuda):
    import oracle

    if oracle.load_ref() is None:
        pytest.skip("reference build not available on this box")
    ref = oracle.RefGallatin(2 << 30, 4, 16 << 20, 128, 4096)
    try:
        heads = cuda.zeros(BUCKETS, dtype=cuda.int64, device="cuda")
        st = zeros(cuda)
        ref.table_op(heads.data_ptr(), BUCKETS, 9, gal.TABLE_OPS["insert"], N, st.data_ptr())
        ref.table_op(heads.data_ptr(), BUCKETS, 9, gal.TABLE_OPS["query"], N, st.data_ptr())
        s = read(cuda, st)
        assert s[0] == 0 and s[1] == 0 and s[2] == 0
        ref.table_op(heads.data_ptr(), BUCKETS, 9, gal.TABLE_OPS["clear"], 0, st.data_ptr())
        lengths = vector_lengths(1 << 14, seed=6)
        d_len = cuda.from_numpy(lengths.view(np.int32)).cuda()
        st = zeros(cuda)
        ref.run_vectors(d_len.data_ptr(), len(lengths), st.data_ptr())
        s = read(cuda, st)
        assert s[0] == 0 and s[2] == 0 and s[4] == int(lengths.sum())
    finally:
        ref.close()

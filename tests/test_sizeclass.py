"""Size classing and allocation sizes against a restatement of the reference dispatch (CPU only)."""
from __future__ import annotations

import numpy as np
import pytest

import gallatin_gb300 as gal


def first_bit_bigger(v: int) -> int:
    """alloc_utils.cuh:382-398: 63 - clz(v) + (popc(v) != 1)."""
    return (v.bit_length() - 1) + (bin(v).count("1") != 1)


def reference_dispatch(size: int, smallest: int, biggest: int, seg: int):
    """gallatin.cuh:1141-1147 (get_tree_id_from_size) and 1196-1260 (malloc)."""
    smallest_bits = first_bit_bigger(smallest)
    num_trees = first_bit_bigger(biggest) - smallest_bits + 1
    tree_id = 0 if size < smallest else first_bit_bigger(size) - smallest_bits
    if tree_id >= num_trees:
        smallest_tree_bits = first_bit_bigger(smallest * 4096)
        block_tree = first_bit_bigger(size) - smallest_tree_bits
        if block_tree < 0:
            return ("slice", num_trees - 1, 1 << (tree_id - (num_trees - 1)))
        if block_tree < num_trees:
            return ("block", block_tree, 1)
        return ("segment", 0, (size - 1) // seg + 1)
    return ("slice", tree_id, 1)


GEOMS = [(16, 4096, 16 << 20), (128, 4096, 16 << 20), (16, 4096, 64 << 20), (16, 1024, 4 << 20), (32, 2048, 8 << 20)]


@pytest.mark.parametrize("smallest,biggest,seg", GEOMS)
def test_classify_matches_reference_dispatch(smallest, biggest, seg):
    rng = np.random.default_rng(0)
    sizes = list(range(0, 70000, 7)) + [1 << k for k in range(40)] + [(1 << k) + 1 for k in range(40)]
    sizes += [int(x) for x in rng.integers(1, 1 << 36, size=5000)]
    for s in sizes:
        want = reference_dispatch(s, smallest, biggest, seg)
        got = gal.classify(s, smallest, biggest, seg)
        assert got == want, (s, got, want)


def test_default_geometry_tiers():
    assert gal.classify(16) == ("slice", 0, 1)
    assert gal.classify(17) == ("slice", 1, 1)
    assert gal.classify(4096) == ("slice", 8, 1)
    assert gal.classify(8192) == ("slice", 8, 2)  # an 8 KiB page: two 4 KiB slices
    assert gal.classify(32 << 10) == ("slice", 8, 8)
    assert gal.classify((32 << 10) + 1) == ("block", 0, 1)
    assert gal.classify(16 << 20) == ("block", 8, 1)
    assert gal.classify((16 << 20) + 1) == ("segment", 0, 2)
    assert gal.classify(256 << 20) == ("segment", 0, 16)


def test_vector_lengths_shape():
    from gallatin_gb300.workload import vector_lengths

    v = vector_lengths()  # the benchmark's 1M vectors
    assert v.dtype == np.uint32 and v.min() >= 1 and v.max() <= 65536
    assert 60 <= int(np.median(v)) <= 68  # median 64
    assert (v == 65536).sum() >= 1  # the cap is reached (sigma 1.5)

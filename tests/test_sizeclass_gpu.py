"""Device size classing against a restatement of the reference's dispatch.

gal_size_classes runs the device `classify` and `allocated_size` that
malloc and the drop-in header use over a list of request sizes. Their
results must equal the reference's malloc dispatch (gallatin.cuh:1141-1147,
1196-1260) and get_allocated_size (gallatin.cuh:1152-1183) restated below,
quirks included: get_allocated_size only moves to whole segments when both
the slice tree id and the block tree id exceed num_trees (strictly), and
requests under 16 B count as 16 B whatever the smallest slice."""
from __future__ import annotations

import numpy as np
import pytest

import gallatin_gb300 as gal
from test_sizeclass import GEOMS, first_bit_bigger, reference_dispatch

pytestmark = pytest.mark.gpu

M64 = (1 << 64) - 1


def reference_allocated_size(size: int, smallest: int, biggest: int, seg: int) -> int:
    """gallatin.cuh:1152-1183, with the reference's integer widths (bit_size and
    tree_size are uint16_t, the results wrap at 2^64)."""
    if size < 16:
        size = 16
    smallest_bits = first_bit_bigger(smallest)
    num_trees = first_bit_bigger(biggest) - smallest_bits + 1
    smallest_tree_bits = first_bit_bigger(smallest * 4096)
    bit_size = first_bit_bigger(size) & 0xFFFF
    tree_size = 0 if size < smallest else (first_bit_bigger(size) - smallest_bits) & 0xFFFF
    if tree_size > num_trees:
        block_tree = bit_size - smallest_tree_bits
        if block_tree > num_trees:
            return (((size - 1) // seg + 1) * seg) & M64
    return (1 << bit_size) & M64


def request_sizes(seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    sizes = list(range(0, 70000, 7)) + [1 << k for k in range(64)] + [(1 << k) + 1 for k in range(63)]
    sizes += [(1 << k) - 1 for k in range(1, 65)]
    sizes += [int(x) for x in rng.integers(1, 1 << 36, size=4000)]
    sizes += [int(x) for x in rng.integers(1, 1 << 62, size=500, dtype=np.int64)] + [M64, M64 - 1, 1 << 63]
    return np.array(sizes, dtype=np.uint64)


@pytest.mark.parametrize("smallest,biggest,seg", GEOMS)
def test_device_classify_and_allocated_size_match_reference(cuda, smallest, biggest, seg):
    sizes = request_sizes()
    with gal.Gallatin.generate_on_device(4 * seg, 1, print_info=False, segment_size=seg, min_size=smallest,
                                         max_size=biggest) as a:
        d_sizes = cuda.from_numpy(sizes.view(np.int64)).cuda()
        d_out = cuda.zeros(len(sizes) * gal.SIZE_INFO_DTYPE.itemsize, dtype=cuda.uint8, device="cuda")
        a.size_classes(d_sizes.data_ptr(), len(sizes), d_out.data_ptr())
        cuda.cuda.synchronize()
        got = d_out.cpu().numpy().view(gal.SIZE_INFO_DTYPE)
    for s, g in zip(sizes.tolist(), got):
        want = reference_dispatch(s, smallest, biggest, seg)
        have = (gal.TIERS[int(g["tier"])], int(g["tree"]), int(g["count"]))
        assert have == want, f"size {s}: device dispatch {have}, reference {want}"
        want_bytes = reference_allocated_size(s, smallest, biggest, seg)
        assert int(g["allocated"]) == want_bytes, f"size {s}: device allocated {int(g['allocated'])}, want {want_bytes}"

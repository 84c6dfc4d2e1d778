"""Batched find-at-or-after on the GPU (gal_veb_find_batch): the staged form
(each CTA copies the tree's upper layers into shared memory) and the
global-memory form both give, for every query, the smallest set id at or
after it, checked against a brute-force model on trees loaded with
gal_veb_load, including trees whose upper layers do not all fit the staging
budget."""
from __future__ import annotations

import numpy as np
import pytest

import gallatin_gb300 as gal

pytestmark = pytest.mark.gpu

FAIL = np.uint64(~np.uint64(0))


def leaf_words(universe: int, ids: np.ndarray) -> np.ndarray:
    words = np.zeros((universe - 1) // 64 + 1, dtype=np.uint64)
    np.bitwise_or.at(words, ids >> 6, np.left_shift(np.uint64(1), (ids & 63).astype(np.uint64)))
    return words


def model(universe: int, ids: np.ndarray, q: np.ndarray) -> np.ndarray:
    ids = np.sort(ids)
    pos = np.searchsorted(ids, q, side="left")
    out = np.full(len(q), FAIL, dtype=np.uint64)
    hit = (pos < len(ids)) & (q < np.uint64(universe))
    out[hit] = ids[pos[hit]]
    return out


def upper_layers(words: np.ndarray, layers: int) -> list[np.ndarray]:
    """Every layer of a consistent tree, leaf last: each upper bit is set when
    its child word holds a set bit."""
    out = [words]
    for _ in range(layers - 1):
        child = out[0]
        parent = np.zeros((len(child) - 1) // 64 + 1, dtype=np.uint64)
        nz = np.nonzero(child)[0].astype(np.uint64)
        np.bitwise_or.at(parent, nz >> 6, np.left_shift(np.uint64(1), (nz & 63).astype(np.uint64)))
        out.insert(0, parent)
    return out


@pytest.mark.parametrize("universe,density", [
    (1, 1.0), (63, 0.5), (64, 0.0), (65, 1.0), (4097, 0.01), (262145, 1 / 256), (262145, 0.5),
    ((1 << 22) + 3, 1 / 4096), ((1 << 26) + 5, 1 / 256),
])
def test_batched_find_matches_a_brute_force_model(cuda, universe, density):
    rng = np.random.default_rng(universe ^ int(density * 1e6))
    k = int(universe * density)
    ids = np.unique(rng.integers(0, universe, size=k, dtype=np.uint64)) if k else np.zeros(0, dtype=np.uint64)
    if density == 1.0:
        ids = np.arange(universe, dtype=np.uint64)
    n = 1 << 20 if universe > 4096 else 4096
    q = rng.integers(0, universe + 100, size=n, dtype=np.uint64)
    edges = np.array([0, universe - 1, universe, universe + 1], dtype=np.uint64)
    q = np.concatenate([q, edges, ids[:1000], ids[:1000] + np.uint64(1)])
    want = model(universe, ids, q)
    words = leaf_words(universe, ids)
    with gal.VebTree(universe, 3) as tree:
        tree.load(words)
        got_layers = tree.layers()
        for a, b in zip(got_layers, upper_layers(words, len(got_layers))):
            assert np.array_equal(a, b), "loaded layers are not the OR of their children"
        d_q = cuda.from_numpy(q.view(np.int64)).cuda()
        for staged in (True, False):
            d_out = cuda.full((len(q),), -7, dtype=cuda.int64, device="cuda")
            tree.find_batch(d_q.data_ptr(), len(q), d_out.data_ptr(), staged=staged)
            cuda.cuda.synchronize()
            got = d_out.cpu().numpy().view(np.uint64)
            bad = np.nonzero(got != want)[0]
            assert len(bad) == 0, (staged, int(q[bad[0]]), int(got[bad[0]]), int(want[bad[0]]))


def test_load_rejects_bits_past_the_universe(cuda):
    with gal.VebTree(100, 1) as tree:
        words = np.zeros(2, dtype=np.uint64)
        words[1] = np.uint64(1) << np.uint64(40)  # id 104
        with pytest.raises(gal.GalError):
            tree.load(words)
        with pytest.raises(gal.GalError):
            tree.load(np.zeros(3, dtype=np.uint64))

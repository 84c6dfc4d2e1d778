"""vEB parity on the GPU: the device tree against the reference's golden vectors,
the oracle, and (when built on this machine) the reference's own veb_tree."""
from __future__ import annotations

import numpy as np
import pytest

import gallatin_gb300 as gal
import oracle

pytestmark = pytest.mark.gpu


def run_device(torch, universe: int, seed: int, ops: np.ndarray):
    with gal.VebTree(universe, seed) as tree:
        d_ops = torch.from_numpy(np.ascontiguousarray(ops).view(np.uint8).copy()).cuda()
        d_res = torch.zeros(len(ops), dtype=torch.int64, device="cuda")
        tree.run_ops(d_ops.data_ptr(), len(ops), d_res.data_ptr())
        torch.cuda.synchronize()
        return d_res.cpu().numpy().view(np.uint64).copy(), tree.layers()


def test_single_bit_ops_match_reference_golden(cuda, golden):
    """insert / insert_force_update / remove / query / successor(_thorough) /
    lock_offset / malloc_first / find_first / find_random / malloc: bit-exact
    results and final layers against the reference run on a GB300."""
    for s in golden:
        if s["kind"] != "single":
            continue
        res, layers = run_device(cuda, s["universe"], s["seed"], s["ops"])
        bad = np.nonzero(res != s["results"])[0]
        assert bad.size == 0, f"set {s['index']} U={s['universe']}: first mismatch at op {bad[:1]}"
        for got, want in zip(layers, s["layers"]):
            assert np.array_equal(got, want)


def test_run_ops_match_gb300_oracle_exactly(cuda, golden):
    for s in golden:
        res, layers = run_device(cuda, s["universe"], s["seed"], s["ops"])
        want, want_layers, _ = oracle.veb_run(s["universe"], s["seed"], oracle.MODE_GB300, s["ops"])
        bad = np.nonzero(res != want)[0]
        assert bad.size == 0, f"set {s['index']}: first mismatch at op {bad[:1]}"
        for got, w in zip(layers, want_layers):
            assert np.array_equal(got, w)


def test_run_ops_match_reference_until_its_first_quirk(cuda, golden):
    for s in golden:
        if s["kind"] != "runs":
            continue
        _, _, quirks = oracle.veb_run(s["universe"], s["seed"], oracle.MODE_REFERENCE, s["ops"])
        first_quirk = int(np.argmax(quirks > 0)) if quirks[-1] > 0 else len(quirks)
        res, _ = run_device(cuda, s["universe"], s["seed"], s["ops"])
        assert np.array_equal(res[:first_quirk], s["results"][:first_quirk])


@pytest.mark.parametrize("universe", [1, 64, 4097, 70000])
def test_live_differential_against_reference_build(cuda, universe):
    """Fresh seeded sets run on the reference veb_tree built on this machine and on
    the GB300 tree side by side."""
    if oracle.load_ref() is None:
        pytest.skip("reference build not available on this box")
    rng = np.random.default_rng(universe)
    n = 1500
    ops = np.zeros(n, dtype=oracle.VEB_OP_DTYPE)
    ops["code"] = rng.choice([0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 13], size=n)
    ops["arg"] = rng.integers(0, universe, size=n, dtype=np.uint64)
    ops["tid"] = rng.integers(0, 1024, size=n, dtype=np.uint32)
    ref = oracle.RefVeb(universe, 11)
    try:
        d_ops = cuda.from_numpy(ops.view(np.uint8).copy()).cuda()
        d_res = cuda.zeros(n, dtype=cuda.int64, device="cuda")
        ref.run_ops(d_ops.data_ptr(), n, d_res.data_ptr())
        cuda.cuda.synchronize()
        want = d_res.cpu().numpy().view(np.uint64).copy()
        want_layers = ref.layers()
    finally:
        ref.close()
    got, got_layers = run_device(cuda, universe, 11, ops)
    assert np.array_equal(got, want)
    for a, b in zip(got_layers, want_layers):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("universe", [1, 64, 65, 127, 4097, 70000, 300000])
def test_allocator_searches_match_a_brute_force_model(cuda, universe):
    """The allocator's own searches (find_at_or_after, claim_first) on a tree
    changed only by insert_force_update and remove (as the allocator's are):
    every answer equals the smallest set id >= the argument in a set model,
    including leaf words read in pairs past odd word counts, and the layers
    end equal to the oracle's for the same insert/remove sequence."""
    rng = np.random.default_rng(universe + 5)
    n = 3000
    ops = np.zeros(n, dtype=oracle.VEB_OP_DTYPE)
    ops["code"] = rng.choice([1, 2, 14, 15], size=n, p=[0.35, 0.35, 0.25, 0.05])
    ops["arg"] = rng.integers(0, universe, size=n, dtype=np.uint64)
    # a third of the searches start at the last bit of a word
    edge = rng.random(n) < 0.33
    ops["arg"][edge] = np.minimum(
        (rng.integers(0, max(universe // 64, 1), size=int(edge.sum())) * 64 + 63).astype(np.uint64),
        np.uint64(universe - 1))
    # thin the full tree first so the searches cross empty words and layers
    pre = np.zeros(universe, dtype=oracle.VEB_OP_DTYPE)
    pre["code"] = 2
    pre["arg"] = np.arange(universe, dtype=np.uint64)
    keep = rng.random(universe) < 0.05
    pre = pre[~keep]
    seq = np.concatenate([pre, ops])
    res, layers = run_device(cuda, universe, 3, seq)
    present = np.ones(universe, dtype=bool)  # the tree starts full
    fail = np.uint64((1 << 64) - 1)
    for i, op in enumerate(seq):
        code, arg = int(op["code"]), int(op["arg"])
        got = res[i]
        if code == 1:
            assert bool(got) == (not present[arg])
            present[arg] = True
        elif code == 2:
            assert bool(got) == bool(present[arg])
            present[arg] = False
        else:
            start = 0 if code == 15 else arg
            idx = np.flatnonzero(present[start:])
            want = np.uint64(start + idx[0]) if idx.size else fail
            assert got == want, f"op {i} ({code}, {arg}): got {int(got)}, want {int(want)}"
            if code == 15 and idx.size:
                present[start + idx[0]] = False
    # the final layers equal the oracle's after the same inserts and removes
    # (each successful claim is a remove of the id it returned)
    claims = seq["code"] == 15
    model_ops = seq.copy()
    model_ops["code"][claims] = 2
    model_ops["arg"][claims] = res[claims]
    model_ops = model_ops[(model_ops["code"] != 14) & ~(claims & (res == fail))]
    _, want_layers, _ = oracle.veb_run(universe, 3, oracle.MODE_GB300, model_ops)
    for got, want in zip(layers, want_layers):
        assert np.array_equal(got, want)

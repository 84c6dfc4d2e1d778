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

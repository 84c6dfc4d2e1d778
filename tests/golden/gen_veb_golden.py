#!/usr/bin/env python3
"""Generate tests/golden/veb_golden.npz from the REFERENCE vEB tree on a GPU.

Seeded, ordered op sequences are run through the reference's own veb_tree
(saltsystemslab/gallatin include/gallatin/allocators/veb.cuh, compiled
unmodified into oracle/_ref/libgalref_core.so by oracle/build.py) with the
single-block op runner of oracle/ref_core.cu: op i executes on thread
ops[i].tid, so the hashed ops (find_random_valid_index, malloc) see that
thread id. The fixture stores, per sequence, the ops, every op's result and
the final bit layers. Needs a GPU, torch and the staged reference headers.

Two families:
  single  insert / insert_force_update / remove / query / successor /
          successor_thorough / lock_offset / malloc_first /
          find_first_valid_index / find_random_valid_index / malloc /
          report_fill on many universe sizes (1 .. 262145, 1-4 layers)
  runs    segment-tree style sequences adding gather_multiple (n <= 64, the
          range where the reference stays in bounds) and return_multiple of
          previously gathered runs; arguments are chosen by replaying the
          oracle, which only steers the choice of valid arguments.

usage: python tests/golden/gen_veb_golden.py [--out PATH]
"""
from __future__ import annotations

import argparse
import sys
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(REPO))

import oracle  # noqa: E402
from oracle import VEB_OP_DTYPE  # noqa: E402

UNIVERSES_SINGLE = [1, 2, 63, 64, 65, 127, 128, 129, 512, 4095, 4096, 4097, 7680, 262144, 262145]
UNIVERSES_RUNS = [64, 65, 128, 129, 512, 4097, 7680]
FAIL = (1 << 64) - 1


def single_ops(universe: int, rng: np.random.Generator, n: int, thin_frac: float = 0.4) -> np.ndarray:
    ops = np.zeros(n, dtype=VEB_OP_DTYPE)
    thin = ([2, 6, 7, 10, 3, 4, 9], [0.55, 0.1, 0.1, 0.1, 0.05, 0.05, 0.05])
    mixed = (
        [0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 13],
        [0.06, 0.14, 0.2, 0.1, 0.1, 0.1, 0.06, 0.04, 0.03, 0.09, 0.06, 0.02],
    )
    split = int(thin_frac * n)
    ops["code"][:split] = rng.choice(thin[0], size=split, p=thin[1])
    ops["code"][split:] = rng.choice(mixed[0], size=n - split, p=mixed[1])
    ops["arg"] = rng.integers(0, universe, size=n, dtype=np.uint64)
    ops["tid"] = rng.integers(0, 1024, size=n, dtype=np.uint32)
    return ops


def runs_ops(universe: int, seed: int, rng: np.random.Generator, n: int) -> np.ndarray:
    codes = [7, 11, 12, 99, 2, 1, 5, 3, 6, 13]  # 99: return of a random range
    probs = [0.2, 0.25, 0.15, 0.05, 0.1, 0.1, 0.05, 0.03, 0.04, 0.03]
    ops = np.zeros(0, dtype=VEB_OP_DTYPE)
    outstanding: list[tuple[int, int]] = []
    chunk = 40
    max_run = min(64, universe)
    while len(ops) < n:
        new = np.zeros(chunk, dtype=VEB_OP_DTYPE)
        gathers = []
        for i in range(chunk):
            code = int(rng.choice(codes, p=probs))
            tid = int(rng.integers(0, 1024))
            arg = int(rng.integers(0, universe))
            arg2 = 0
            if code == 11:
                arg = int(min(max_run, max(1, int(rng.exponential(8)))))
                gathers.append((i, arg))
            elif code == 12:
                if outstanding:
                    start, length = outstanding.pop(int(rng.integers(0, len(outstanding))))
                    arg, arg2 = start, length
                else:
                    code, arg = 7, 0
            elif code == 99:
                code = 12
                arg = int(rng.integers(0, universe))
                arg2 = int(rng.integers(1, min(64, universe - arg) + 1))
            new[i] = (code, tid, arg, arg2)
        base = len(ops)
        ops = np.concatenate([ops, new])
        results, _, _ = oracle.veb_run(universe, seed, oracle.MODE_REFERENCE, ops)
        for i, length in gathers:
            r = int(results[base + i])
            if r < FAIL - 2:
                outstanding.append((r, length))
    return ops[:n]


def build_sets():
    sets = []
    for k, u in enumerate(UNIVERSES_SINGLE):
        rng = np.random.default_rng(1000 + k)
        n = 300 if u < 8 else 2000
        seed = 42 + k
        sets.append(("single", u, seed, single_ops(u, rng, n)))
    for k, u in enumerate([4096, 7680]):  # thinned large trees: long successor walks
        rng = np.random.default_rng(3000 + k)
        sets.append(("single", u, 99 + k, single_ops(u, rng, 6000, thin_frac=0.7)))
    for k, u in enumerate(UNIVERSES_RUNS):
        rng = np.random.default_rng(5000 + k)
        seed = 7 + k
        sets.append(("runs", u, seed, runs_ops(u, seed, rng, 1500)))
    return sets


def run_reference(universe: int, seed: int, ops: np.ndarray):
    import torch

    tree = oracle.RefVeb(universe, seed)
    try:
        d_ops = torch.from_numpy(ops.view(np.uint8).copy()).cuda()
        d_res = torch.zeros(len(ops), dtype=torch.int64, device="cuda")
        tree.run_ops(d_ops.data_ptr(), len(ops), d_res.data_ptr())
        torch.cuda.synchronize()
        results = d_res.cpu().numpy().view(np.uint64).copy()
        layers = tree.layers()
    finally:
        tree.close()
    return results, layers


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=str(REPO / "tests" / "golden" / "veb_golden.npz"))
    args = ap.parse_args()
    if oracle.load_ref() is None:
        print("reference build unavailable (stage the reference headers and build oracle/_ref first)")
        return 1
    payload = {}
    kinds, universes, seeds = [], [], []
    for i, (kind, u, seed, ops) in enumerate(build_sets()):
        results, layers = run_reference(u, seed, ops)
        payload[f"s{i}_ops"] = ops
        payload[f"s{i}_results"] = results
        payload[f"s{i}_layers"] = np.concatenate(layers)
        payload[f"s{i}_layer_words"] = np.array([len(x) for x in layers], dtype=np.int64)
        kinds.append(0 if kind == "single" else 1)
        universes.append(u)
        seeds.append(seed)
        print(f"set {i}: {kind} U={u} ops={len(ops)} layers={[len(x) for x in layers]}")
    payload["kind"] = np.array(kinds, dtype=np.int64)
    payload["universe"] = np.array(universes, dtype=np.uint64)
    payload["seed"] = np.array(seeds, dtype=np.uint64)
    out = Path(args.out)
    out.parent.mkdir(parents=True, exist_ok=True)
    np.savez_compressed(out, **payload)
    print(f"wrote {out} ({out.stat().st_size} bytes)")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())

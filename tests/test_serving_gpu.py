"""Serving loop on the GPU: admission as the host model says, every finished
stream's checksum equal to the oracle's (its pages were its own while it
lived), the same result for a stream alone and in the mix, both launch forms
agreeing, and the allocator restored after the drain."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import gallatin_gb300 as gal
import oracle
from alloc_checks import check_restored
from gallatin_gb300.serving import NOT_SET, ServingRun, summarize
from gallatin_gb300.workload import serving_admission, serving_trace, single_stream

pytestmark = pytest.mark.gpu

ARENA = 2 << 30
BUDGET = int(0.8 * (1 << 30)) // 8192  # the gate binds well inside the arena
SLOTS = 4096


def small(seed=3):
    return serving_trace(seed, steps=60, arrivals_per_step=30)


def run_once(cuda, trace, persistent, seed=5):
    with gal.Gallatin.generate_on_device(ARENA, seed, print_info=False) as a:
        run = ServingRun(cuda, trace, budget_pages=BUDGET, max_slots=SLOTS)
        run.run(a.run_serving, persistent=persistent)
        res = run.results()
        a.flush_pinned()
        cuda.cuda.synchronize()
        check_restored(a)
    return res


@pytest.mark.parametrize("persistent", [False, True])
def test_serving_follows_the_admission_model(cuda, persistent):
    tr = small()
    res = run_once(cuda, tr, persistent)
    st = res["step_stats"]
    assert st[:, 7].sum() == 0, "a page malloc returned NULL"
    admit, model = serving_admission(tr, BUDGET, SLOTS)
    assert np.array_equal(res["admit_step"], admit)
    assert np.array_equal(st[:, 4].astype(np.int64), model["committed"])
    assert model["committed"].max() > 0.9 * BUDGET  # the gate was exercised
    adm = admit != NOT_SET
    fin_want = np.where(adm, admit.astype(np.int64) + tr["pages"] - 1, -1)
    fin = res["finish_step"] != NOT_SET
    assert np.array_equal(fin, adm & (fin_want < tr["steps"]))
    assert np.array_equal(res["finish_step"][fin].astype(np.int64), fin_want[fin])
    want = oracle.serving_checksums(tr["tokens"], 42)
    assert np.array_equal(res["checksum"][fin], want[fin])
    assert (res["checksum"][~fin] == 0).all()
    # live pages never exceed what was committed
    assert np.all(st[:, 3] <= st[:, 4])
    s = summarize(res, page_bytes=8192, segment_bytes=16 << 20)
    assert s["latency_ns"]["samples"] == s["pages_allocated"] == int(st[:, 0].sum())
    assert 0.0 <= s["fragmentation"]["at_peak_live"] < 1.0


def test_both_launch_forms_agree(cuda):
    tr = small(4)
    a = run_once(cuda, tr, False)
    b = run_once(cuda, tr, True)
    for k in ("checksum", "admit_step", "finish_step"):
        assert np.array_equal(a[k], b[k]), k
    assert np.array_equal(a["step_stats"][:, :6], b["step_stats"][:, :6])


def test_each_stream_same_alone_and_in_the_mix(cuda):
    tr = small(6)
    mix = run_once(cuda, tr, True)
    fin = np.flatnonzero(mix["finish_step"] != NOT_SET)
    by_len = fin[np.argsort(tr["pages"][fin])]
    picks = [int(by_len[0]), int(by_len[len(by_len) // 2]), int(by_len[-1])]
    want = oracle.serving_checksums(tr["tokens"], 42)
    for i in picks:
        alone = run_once(cuda, single_stream(tr, i), True)
        assert alone["finish_step"][0] == tr["pages"][i] - 1
        assert alone["checksum"][0] == mix["checksum"][i] == want[i], i


def test_serving_rejects_bad_parameters(cuda):
    tr = small(7)
    with gal.Gallatin.generate_on_device(1 << 30, 1, print_info=False) as a:
        run = ServingRun(cuda, tr, budget_pages=BUDGET, max_slots=SLOTS)
        p = run.params()
        p.width = 12
        with pytest.raises(gal.GalError):
            a.run_serving(ctypes.byref(run.c_trace), ctypes.byref(p), ctypes.byref(run.c_out))
        with pytest.raises(ValueError):
            ServingRun(cuda, tr, budget_pages=BUDGET, max_pages=4)


def test_pages_spill_to_a_host_arena_with_the_same_results(cuda):
    # the live pages peak near 226 MiB, well past the 64 MiB device arena:
    # through the fused calls the pages that do not fit land in a host arena,
    # no malloc fails, and every stream's admission, finish and checksum are
    # those of a run on a device arena large enough for all of it
    tr = small(8)
    want = run_once(cuda, tr, True)
    dev = gal.Gallatin.generate_on_device(64 << 20, 5, print_info=False)
    host = gal.Gallatin.generate_on_device_host(1 << 30, 6, print_info=False)
    try:
        run = ServingRun(cuda, tr, budget_pages=BUDGET, max_slots=SLOTS)
        run.run(lambda *a: dev.run_serving_fused(host, *a), persistent=True)
        res = run.results()
        assert res["step_stats"][:, 7].sum() == 0, "a page malloc returned NULL"
        for k in ("checksum", "admit_step", "finish_step"):
            assert np.array_equal(res[k], want[k]), k
        assert host.stats()["counters"]["block_pins"] > 0, "nothing spilled to the host arena"
        assert dev.stats()["counters"]["nomem"] > 0
        for a in (dev, host):
            a.flush_pinned()
            cuda.cuda.synchronize()
            check_restored(a)
    finally:
        dev.free_on_device()
        host.free_on_device()

"""Serving configuration on the CPU: the stream trace, the admission model the
device loop must reproduce, the checksum oracle and the glibc replay."""
from __future__ import annotations

import numpy as np

import oracle
from gallatin_gb300.serving import HIST_BUCKETS, bucket_lower_ns, quantile_ns
from gallatin_gb300.workload import serving_admission, serving_trace, single_stream

M64 = (1 << 64) - 1


def _token(seed, i, p):
    x = (seed ^ ((i << 16) | p)) & M64
    x = (x + 0x9E3779B97F4A7C15) & M64
    x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & M64
    x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & M64
    return x ^ (x >> 31)


def test_trace_shape():
    tr = serving_trace(3, steps=50, arrivals_per_step=20)
    n = len(tr["pages"])
    assert tr["arrivals_end"][0] == 0 and tr["arrivals_end"][-1] == n
    assert np.all(np.diff(tr["arrival_step"].astype(np.int64)) >= 0)
    assert tr["tokens"].min() >= 128 and tr["tokens"].max() <= 32768
    assert np.array_equal(tr["pages"], (tr["tokens"] + 15) // 16)
    assert tr["page_prefix"][-1] == tr["pages"].sum()
    # arrivals_end[s + 1] counts streams that arrived at steps <= s
    for s in (0, 10, 49):
        assert tr["arrivals_end"][s + 1] == np.count_nonzero(tr["arrival_step"] <= s)


def test_admission_model_keeps_its_rules():
    tr = serving_trace(4, steps=80, arrivals_per_step=30)
    budget, slots = 40000, 1500
    admit, st = serving_admission(tr, budget, slots)
    adm = admit != 0xFFFFFFFF
    # first come first served: the admitted streams are a prefix, in order
    k = int(adm.sum())
    assert adm[:k].all() and not adm[k:].any()
    assert np.all(np.diff(admit[:k].astype(np.int64)) >= 0)
    # nobody is admitted before arriving
    assert np.all(admit[:k] >= tr["arrival_step"][:k])
    pages = tr["pages"].astype(np.int64)
    for s in range(tr["steps"]):
        running = adm & (admit <= s) & (admit.astype(np.int64) + pages - 1 >= s)
        assert pages[running].sum() <= budget
        # a slot stays taken one step past its stream's last page (its pages
        # are freed in that step)
        holding = adm & (admit <= s) & (admit.astype(np.int64) + pages >= s)
        assert holding.sum() <= slots
        assert st["committed"][s] == pages[running].sum()
    # the budget binds at some step (the gate is exercised)
    assert st["committed"].max() > 0.9 * budget


def test_checksum_oracle_against_python():
    tr = serving_trace(5, steps=10, arrivals_per_step=5)
    got = oracle.serving_checksums(tr["tokens"], 42, 2)
    for i in range(min(6, len(got))):
        want = sum(_token(42, i, p) * (2 * p + 1) for p in range(int(tr["tokens"][i]))) & M64
        assert int(got[i]) == want


def test_glibc_replay_reports_the_oracle_checksums():
    tr = serving_trace(6, steps=40, arrivals_per_step=20)
    admit, _ = serving_admission(tr, 30000, 4096)
    secs, chk, hist, nulls = oracle.cpu_replay_serving(tr, admit, workers=3)
    want = oracle.serving_checksums(tr["tokens"], 42)
    fin = (admit != 0xFFFFFFFF) & (admit.astype(np.int64) + tr["pages"] - 1 < tr["steps"])
    assert fin.any() and nulls == 0
    assert np.array_equal(chk[fin], want[fin])
    assert (chk[~fin] == 0).all()
    assert hist.sum() > 0


def test_single_stream_keeps_its_id():
    tr = serving_trace(7, steps=20, arrivals_per_step=10)
    one = single_stream(tr, 5)
    assert one["ids"][0] == 5 and one["tokens"][0] == tr["tokens"][5]
    assert one["steps"] == int(tr["pages"][5]) + 2
    admit, _ = serving_admission(one, 10**9, 1)
    assert admit[0] == 0


def test_latency_quantiles():
    lo, width = bucket_lower_ns()
    assert len(lo) == HIST_BUCKETS and lo[32] == 32 and lo[64] == 64 and width[64] == 2
    hist = np.zeros(HIST_BUCKETS, dtype=np.uint64)
    hist[100] = 99
    hist[500] = 1
    assert lo[100] <= quantile_ns(hist, 0.5) <= lo[100] + width[100]
    assert lo[500] <= quantile_ns(hist, 1.0) <= lo[500] + width[500]

#!/usr/bin/env python3
"""Benchmark: malloc+free pairs per second of the device allocator on GB300.

Default workload (the reference metric's mixed-size configuration): an 8 GiB
arena of 16 MiB segments, Gallatin<16 MiB, 16, 4096>; 4,194,304 threads, each
for 8 rounds mallocs 16 << k bytes (k = x mod 9 of a per-thread xorshift64
seeded by splitmix64(42 + tid)), fills every 16 bytes with tid ^ round,
verifies and frees; plus 256 segment-tier requests of 16-256 MiB (thread 0
of every 64th 256-thread CTA). One step = one launch of that workload kernel.
`--workload pairs` runs the small plain configuration instead: a 2 GiB arena,
1,048,576 threads (1024 x 1024), malloc 16 B / store tid / verify / free.
The other workloads (batches, table, vectors, serving, spill, calloc) are
described where WORKLOADS defines them.

value: pairs/s with the class trace resident in HBM, device time from CUDA
events on the launching stream, L2 flushed (256 MiB write) before every
timed step. e2e: the same metric through the C-ABI host-buffer entry point
(gal_run_mixed_host): the pinned host class trace is copied to the device,
the kernel runs, the stats words come back, all inside the timed region.

--impl reference runs the reference's own CUDA build (oracle/_ref, the
reference headers compiled for sm_103a) through the same workload kernels.
Under torchrun every rank runs an independent replica (the allocator is one
arena per GPU: replicas only, no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO))

GIB = 1 << 30
MIB = 1 << 20
REF_BATCH_PREFIX = 40
# The reference allocator serves the serving trace's first 150 steps, but on
# the full 600-step trace back-to-back runs exhaust its arena (blocks are
# recycled only once every slice is back): by the fourth run every page
# malloc returned NULL. Its arm, and a matching line of ours, use 150 steps.
REF_SERVE_STEPS = 150

WORKLOADS = {
    "mixed": dict(
        arena=8 * GIB, segment=16 * MIB, min_size=16, max_size=4096, threads=4_194_304, rounds=8, block=256,
        seg_every=64, seg_lo=16 * MIB, seg_hi=256 * MIB,
    ),
    "pairs": dict(arena=2 * GIB, segment=16 * MIB, min_size=16, max_size=4096, threads=1_048_576, size=16, block=1024),
    # the batching configuration: 64 batches of 1k-512k requests, lognormal
    # sizes, 60/40 malloc/free over the live set, plus a drain batch
    # form: how the stream is served, each captured once in a CUDA graph:
    # "launches" (one launch per batch), "persistent" (one cooperative kernel
    # over all batches) or "binned" (the same, each batch counting-sorted by
    # size class first); --batch-form overrides it
    "batches": dict(arena=8 * GIB, segment=16 * MIB, min_size=16, max_size=4096, batches=64, width=32,
                    form="launches"),
    # the data-structure configuration: a chained hash table of 64M keys
    # (insert all, erase half, reinsert them) with 120 B nodes from a 128 B
    # minimum allocator, and 1M doubling vectors
    "table": dict(arena=32 * GIB, segment=16 * MIB, min_size=128, max_size=4096, keys=1 << 26, buckets=1 << 24),
    "vectors": dict(arena=32 * GIB, segment=16 * MIB, min_size=128, max_size=4096, vectors=1_000_000),
    # the serving configuration: Poisson arrivals (2,000 streams/s at 0.5 s
    # per 16-token step), lognormal lengths, one 8 KiB page per step, the
    # admission gate at 80 % of a 120 GiB arena
    "serving": dict(arena=120 * GIB, segment=16 * MIB, min_size=16, max_size=4096, steps=600, arrivals=1000.0,
                    page_bytes=8192, slots=262144, max_pages=2048, gate=0.8,
                    # one CTA per SM: CTAs left idle in a step wait at the grid
                    # barrier and slow the working ones (measured 1-4 per SM)
                    ctas_per_sm=1),
    # the mixed workload without its 256 segment-tier requests: only the
    # slice tier runs, which is what the reference arm can be compared on
    "mixed-slices": dict(
        arena=8 * GIB, segment=16 * MIB, min_size=16, max_size=4096, threads=4_194_304, rounds=8, block=256,
        seg_every=0, seg_lo=16 * MIB, seg_hi=256 * MIB,
    ),
    # device first, host arena when the device arena is out of room (the
    # reference's global_malloc_fused / global_free_fused): 8,388,608
    # allocations of 16..4096 B (about 7.6 GB) against a 4 GiB device arena
    # and an 8 GiB pinned host arena; one step = a fill launch (malloc, write
    # the first and last u64) and a drain launch (verify, free)
    "spill": dict(arena=4 * GIB, host_arena=8 * GIB, segment=16 * MIB, min_size=16, max_size=4096,
                  threads=8_388_608),
    # the serving loop under memory pressure: the same trace and gate (80 % of
    # all memory) over an 8 GiB device arena and a 16 GiB pinned host arena,
    # every page malloc device-first with the host arena on NULL
    "serving-spill": dict(arena=8 * GIB, host_arena=16 * GIB, segment=16 * MIB, min_size=16, max_size=4096,
                          steps=600, arrivals=1000.0, page_bytes=8192, slots=262144, max_pages=2048, gate=0.8,
                          ctas_per_sm=1),
    # the mixed-slices workload on an allocator that returns zeroed memory
    # (the reference's running_calloc): every free zeroes its slices
    "calloc": dict(
        arena=8 * GIB, segment=16 * MIB, min_size=16, max_size=4096, threads=4_194_304, rounds=8, block=256,
        seg_every=0, seg_lo=16 * MIB, seg_hi=256 * MIB, calloc=True,
    ),
    # batched find-at-or-after on a standalone vEB tree of 2^26 ids, one in
    # 256 set (uniform), 64 M uniform queries; the staged form keeps the upper
    # layers in shared memory, the global form reads every layer from memory
    "veb-find": dict(universe=1 << 26, density=1 / 256, queries=1 << 26),
}


def measured_peaks() -> dict:
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except ValueError:
            pass
    return {}


def l2_atomic_roofline(torch, stream, atomics_per_unit, units_per_s) -> dict:
    """Peak L2 atomic rate of this GPU, measured here with the library's probe
    (single-lane 64-bit atomics, each to its own 128-byte line, 8 in flight per
    warp: the allocator's leader pattern), best of several launches timed with
    CUDA events; and the allocator's achieved rate, atomics_per_unit (an ncu
    count of L2 atomic + reduction requests of the timed kernel, per unit) x
    units per second."""
    import gallatin_gb300 as gal

    buf = torch.zeros(32 * MIB, dtype=torch.uint8, device="cuda")
    best = {}
    for mode, name in ((0, "atom"), (1, "red")):
        for ctas in (4, 8):
            gal.probe_l2_atomics(buf.data_ptr(), buf.numel(), 64, mode, ctas, stream=stream.cuda_stream)  # warm-up
            for _ in range(3):
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                ops = gal.probe_l2_atomics(buf.data_ptr(), buf.numel(), 512, mode, ctas, stream=stream.cuda_stream)
                e1.record(stream)
                e1.synchronize()
                rate = ops / (e0.elapsed_time(e1) / 1e3)
                best[name] = max(best.get(name, 0.0), rate)
    del buf
    out = {"unit": "atomics/s", "peak": best["atom"], "peak_red": best["red"],
           "peak_source": "measured in this run: gal_probe_l2_atomics, single-lane atom.add.u64 to distinct "
                          "128-B lines, best of 3 launches x {4, 8} CTAs/SM",
           "atomics_per_unit": atomics_per_unit, "achieved": None, "frac": None}
    if atomics_per_unit:
        out["achieved"] = atomics_per_unit * units_per_s
        out["frac"] = out["achieved"] / out["peak"]
    return out


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples during the timed region.

    Sampling starts before the region and the sampler waits for its first
    sample, and it keeps sampling for a short while after the region, so a
    region shorter than the 50 ms sampling period (the 16 B pairs workload
    times well under a millisecond) is still bracketed by samples taken
    next to it."""

    QUERY = (
        "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
        "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
        "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"
    )

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []
        self._reader = None

    def _read(self):
        for ln in self.proc.stdout:
            if ln.strip():
                self.lines.append(ln.strip())

    def __enter__(self):
        import threading

        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True,
            )
        except OSError:
            self.proc = None
            return self
        self._reader = threading.Thread(target=self._read, daemon=True)
        self._reader.start()
        t0 = time.perf_counter()
        while not self.lines and time.perf_counter() - t0 < 3.0 and self.proc.poll() is None:
            time.sleep(0.01)
        return self

    def __exit__(self, *exc):
        if self.proc is None:
            return
        n = len(self.lines)
        t0 = time.perf_counter()
        while len(self.lines) < n + 2 and time.perf_counter() - t0 < 1.0 and self.proc.poll() is None:
            time.sleep(0.01)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            self.proc.wait()
        if self._reader is not None:
            self._reader.join(timeout=5)

    def summary(self) -> dict:
        sms, maxes, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sms.append(float(f[1]))
                maxes.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {
            "sm_mhz": statistics.median(sms) if sms else None,
            "sm_max_mhz": max(maxes) if maxes else None,
            "reasons": sorted(reasons),
            "samples": len(sms),
        }


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def barrier_max(torch, world: int, value: float, device: str = "cuda") -> float:
    """The largest of every rank's value (the slowest replica's time)."""
    if world == 1:
        return value
    import torch.distributed as dist

    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units: int, steps: int, world: int, slowest_total_ms: float) -> float:
    """Whole-job throughput of `world` independent replicas that each process
    `units` per step: every replica's work over the slowest replica's time."""
    return units * steps * world / (slowest_total_ms / 1e3)


def barrier(torch, world: int):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def make_allocator(impl: str, w: dict, host: bool = False):
    """The workload's allocator; host=True: the second one, over pinned host
    memory (w["host_arena"] bytes), for the spill workload."""
    size = w["host_arena"] if host else w["arena"]
    seed = 43 if host else 42
    if impl == "reference":
        import oracle

        return oracle.RefGallatin(size, seed, w["segment"], w["min_size"], w["max_size"], host_arena=host)
    import gallatin_gb300 as gal

    if host:
        return gal.Gallatin.generate_on_device_host(size, seed, print_info=False, running_calloc=bool(w.get("calloc")),
                                                    segment_size=w["segment"], min_size=w["min_size"],
                                                    max_size=w["max_size"])
    return gal.Gallatin.generate_on_device(size, seed, print_info=False, running_calloc=bool(w.get("calloc")),
                                           segment_size=w["segment"], min_size=w["min_size"], max_size=w["max_size"],
                                           drop_freed=bool(w.get("drop_freed")))


def close_allocator(impl: str, a) -> None:
    if impl == "reference":
        a.close()
    else:
        a.free_on_device()


def cpu_baseline(name: str, w: dict) -> dict:
    """glibc malloc/free replay of the same trace on this host's cores."""
    import oracle

    cores = os.cpu_count() or 1
    if name == "calloc":
        n, rounds = w["threads"], w["rounds"]
        secs, misses, bad = oracle.cpu_replay_mixed_zeroed(n, 0, n, rounds, 42, workers=cores)
        return {"value": n * rounds / secs, "unit": "malloc+free pairs/s", "cores": cores, "kind": "port",
                "seconds": secs, "misses": misses, "verify_failures": bad,
                "sample": f"full workload: {n} threads x {rounds} rounds through glibc calloc (each allocation "
                          "checked to read zero), fill, verify, free"}
    if name == "spill":
        from gallatin_gb300.workload import mixed_class_trace

        classes = mixed_class_trace(w["threads"], 1, 42).reshape(-1)
        secs, misses, bad = oracle.cpu_replay_fill_drain(classes, cores)
        return {"value": len(classes) / secs, "unit": "malloc+free pairs/s", "cores": cores, "kind": "port",
                "seconds": secs, "misses": misses, "verify_failures": bad,
                "sample": f"full workload: {len(classes)} glibc mallocs (fill), then verify and free (drain); host "
                          "memory has no device arena to spill from"}
    if name in ("mixed", "mixed-slices"):
        n, rounds = w["threads"], w["rounds"]
        secs, misses, bad = oracle.cpu_replay_mixed(
            n, 0, n, rounds, 42, seg_every=w["seg_every"], block_dim=w["block"], seg_lo=w["seg_lo"],
            seg_hi=w["seg_hi"], workers=cores,
        )
        units = n * rounds + (n // w["block"] // w["seg_every"] if w["seg_every"] else 0)
        sample = f"full workload: {n} threads x {rounds} rounds + segment-tier requests, glibc malloc/free"
    elif name == "table":
        secs, bad = oracle.cpu_table(w["keys"], w["buckets"], 9, 42, cores)
        units = w["keys"] * 2
        return {"value": units / secs, "unit": "key ops/s", "cores": cores, "kind": "port", "seconds": secs,
                "misses": bad,
                "sample": f"full workload: {w['keys']} keys insert, half erase, empty-node compaction, half "
                          "reinsert; glibc nodes, atomic CAS, one worker per key range"}
    elif name == "vectors":
        from gallatin_gb300.workload import vector_lengths

        lengths = vector_lengths(w["vectors"])
        secs, bad, pushes = oracle.cpu_vectors(lengths, 1, cores)
        return {"value": pushes / secs, "unit": "pushes/s", "cores": cores, "kind": "port", "seconds": secs,
                "misses": bad,
                "sample": f"full workload: {w['vectors']} vectors grown by doubling with glibc malloc/copy/free"}
    elif name in ("serving", "serving-spill"):
        from gallatin_gb300.serving import quantile_ns
        from gallatin_gb300.workload import serving_admission, serving_trace

        trace = serving_trace(42, steps=w["steps"], arrivals_per_step=w["arrivals"])
        budget = int(w["gate"] * (w["arena"] + w.get("host_arena", 0))) // w["page_bytes"]
        admit, _ = serving_admission(trace, budget, w["slots"])
        secs, checksums, hist, misses = oracle.cpu_replay_serving(trace, admit, page_bytes=w["page_bytes"],
                                                                  workers=cores)
        units = int(hist.sum())
        return {
            "value": units / secs, "unit": "pages/s", "cores": cores, "kind": "port",
            "sample": f"full schedule: {w['steps']} steps, {units} page mallocs, glibc malloc/free, one worker per "
                      "share of the active streams, a barrier per step (the reference has no CPU implementation)",
            "seconds": secs, "misses": misses,
            "latency_ns": {"p50": quantile_ns(hist, 0.5), "p99": quantile_ns(hist, 0.99)},
            "_checksums": checksums,
        }
    elif name == "batches":
        from gallatin_gb300.workload import batch_trace

        reqs, offsets, slots, _ = batch_trace(42, n_batches=w["batches"], batch_hi=w.get("batch_hi", 524288))
        secs, misses = oracle.cpu_replay_batches(reqs, offsets, slots, cores)
        bad = 0
        units = int(offsets[-1])
        sample = f"full request stream: {units} requests in {len(offsets) - 1} batches, glibc malloc/free"
    else:
        n = w["threads"]
        secs, misses, bad = oracle.cpu_replay_pairs(n, w["size"], cores)
        units = n
        sample = f"full workload: {n} threads, glibc malloc/free of {w['size']} B"
    return {
        "value": units / secs,
        "unit": "requests/s" if name == "batches" else "malloc+free pairs/s",
        "cores": cores,
        "kind": "port",
        "sample": sample + " (the reference has no CPU implementation; this replays the trace through glibc)",
        "seconds": secs,
        "misses": misses,
        "verify_failures": bad,
    }


BATCH_FORM_TEXT = {
    "launches": "one launch per batch",
    "persistent": "one persistent cooperative kernel over all batches, warps taking 32 requests at a time",
    "binned": "one persistent cooperative kernel over all batches, each batch counting-sorted by size class on the "
              "device",
}


def batch_form(form: str) -> dict:
    """capture_batches / run_batches arguments of a batch form."""
    return {"persistent": form != "launches", "binned": form == "binned"}


def batch_prefix_rates(torch, a, reqs, offsets, slots, w, stats, flush, steps) -> dict:
    """This allocator on the sample the reference arm of the batching workload
    is timed on (the first batches plus a drain): the configured persistent
    path and the plain one-launch-per-batch path."""
    from gallatin_gb300.workload import prefix_with_drain

    preqs, poffs = prefix_with_drain(reqs, offsets, REF_BATCH_PREFIX)
    n = int(poffs[-1])
    d_reqs = torch.from_numpy(preqs.view(np.int64)).cuda()
    d_offs = torch.from_numpy(poffs.view(np.int64)).cuda()
    d_table = torch.zeros(slots + 1, dtype=torch.int64, device="cuda")
    bargs = (d_reqs.data_ptr(), d_offs.data_ptr(), poffs, d_table.data_ptr(), stats.data_ptr())
    out = {"sample": f"first {REF_BATCH_PREFIX} of {len(offsets) - 2} batches, then a drain batch", "requests": n}
    stream = torch.cuda.current_stream()
    for name, graphed in ((w["form"] + "+graph", True), ("per-thread launches", False)):
        graph = None
        if graphed:
            graph = a.capture_batches(*bargs, width=w["width"], **batch_form(w["form"]))
            fn = lambda: graph.launch(stream.cuda_stream)  # noqa: E731
        else:
            fn = lambda: a.run_batches(*bargs, width=w["width"], persistent=False, stream=stream.cuda_stream)  # noqa: E731
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        stats.zero_()
        times = []
        for _ in range(steps):
            flush.fill_(1)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        if graph is not None:
            graph.close()
        ms = sum(times) / len(times)
        out[name] = {"value": n / (ms / 1e3), "unit": "requests/s", "ms_per_step": ms, "misses": int(stats[0].item())}
    return out


def run_veb_find(args, torch, world, rank, local) -> dict | None:
    """The veb-find workload: one step = one batched search of every query."""
    w = WORKLOADS["veb-find"]
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no batched search: its veb_tree "
                                                                   "answers one successor per call (veb.cuh:836-916)"}))
        return None
    import gallatin_gb300 as gal

    gal.load()
    universe, n = w["universe"], w["queries"]
    rng = np.random.default_rng(42)
    ids = np.unique(rng.integers(0, universe, size=int(universe * w["density"]), dtype=np.uint64))
    words = np.zeros((universe - 1) // 64 + 1, dtype=np.uint64)
    np.bitwise_or.at(words, ids >> np.uint64(6), np.left_shift(np.uint64(1), ids & np.uint64(63)))
    q = rng.integers(0, universe, size=n, dtype=np.uint64)
    stream = torch.cuda.current_stream()
    s_ptr = stream.cuda_stream
    flush = torch.empty(256 * MIB, dtype=torch.uint8, device="cuda")
    d_q = torch.from_numpy(q.view(np.int64)).cuda()
    d_out = torch.empty(n, dtype=torch.int64, device="cuda")
    h_q = torch.from_numpy(q.view(np.int64)).pin_memory()
    h_out = torch.empty(n, dtype=torch.int64).pin_memory()
    # a sample of the answers, from the host model
    sample = np.arange(0, n, 64)
    pos = np.searchsorted(ids, q[sample], side="left")
    want = np.where(pos < len(ids), ids[np.minimum(pos, len(ids) - 1)], np.uint64(~np.uint64(0)))
    forms = {}
    with gal.VebTree(universe, 42) as tree:
        tree.load(words)
        barrier(torch, world)
        with ClockSampler(local) as clocks:
            for staged in (True, False):
                def step():
                    tree.find_batch(d_q.data_ptr(), n, d_out.data_ptr(), staged=staged, stream=s_ptr)

                for _ in range(args.warmup):
                    step()
                torch.cuda.synchronize()
                times = []
                for _ in range(args.steps):
                    flush.fill_(1)
                    ev0 = torch.cuda.Event(enable_timing=True)
                    ev1 = torch.cuda.Event(enable_timing=True)
                    ev0.record(stream)
                    step()
                    ev1.record(stream)
                    ev1.synchronize()
                    times.append(ev0.elapsed_time(ev1))
                got = d_out.cpu().numpy().view(np.uint64)[sample]
                total = barrier_max(torch, world, float(sum(times)))
                forms["staged" if staged else "global"] = {
                    "value": replica_throughput(n, args.steps, world, total), "unit": "queries/s",
                    "ms_per_step": total / args.steps, "step_ms": times,
                    "sample_mismatches": int(np.count_nonzero(got != want))}
            # end to end through the same entry point: queries copied in, answers copied out
            e2e_times = []
            for _ in range(args.steps if not args.no_e2e else 0):
                flush.fill_(1)
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                d_q.copy_(h_q, non_blocking=True)
                tree.find_batch(d_q.data_ptr(), n, d_out.data_ptr(), staged=True, stream=s_ptr)
                h_out.copy_(d_out, non_blocking=True)
                torch.cuda.synchronize()
                e2e_times.append(time.perf_counter() - t0)
    best = forms["staged"]
    ms = best["ms_per_step"]
    alg_bytes = n * 16  # a query read and an answer written; the 8 MiB leaf layer stays in L2
    peak = measured_peaks().get("hbm_gbs") or 6800.0
    achieved = alg_bytes / (ms / 1e3) / 1e9
    result = {
        "metric": "vEB find-at-or-after queries/s (batched, upper layers staged in shared memory)",
        "value": best["value"], "unit": "queries/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic (seeded uniform ids and queries; no dataset)",
        "config": {"workload": f"batched find-at-or-after: universe {universe}, {len(ids)} set ids "
                               f"(density {w['density']:.5f}), {n} uniform queries", "universe": universe,
                   "set_ids": int(len(ids)), "queries": n, "seed": 42,
                   "l2": "inputs and outputs (1 GiB) larger than L2; 256 MiB flush before every timed step"},
        "impl": "gb300",
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None, "algorithmic_bytes_per_launch": alg_bytes,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)"},
        "e2e": None if not e2e_times else {
            "value": replica_throughput(n, args.steps, world, barrier_max(torch, world, sum(e2e_times)) * 1e3),
            "unit": "queries/s", "h2d_bytes_per_step": n * 8, "d2h_bytes_per_step": n * 8,
            "ms_per_step": 1e3 * sum(e2e_times) / len(e2e_times)},
        "clocks": clocks.summary(),
        "gpu_launches": args.steps,
        "misses": 0,
        "verify_failures": forms["staged"]["sample_mismatches"] + forms["global"]["sample_mismatches"],
        "forms": forms,
        "step_ms": best["step_ms"],
    }
    return result if rank == 0 else None


def run(args) -> dict | None:
    import torch

    world, rank, local = dist_setup()
    if args.workload == "veb-find":
        if args.impl == "reference":
            return run_veb_find(args, None, world, rank, local)
        if world > 1:
            torch.cuda.set_device(local)
            import torch.distributed as dist

            dist.init_process_group("nccl")
        else:
            torch.cuda.set_device(local)
        return run_veb_find(args, torch, world, rank, local)
    if args.impl == "reference" and world > 1:
        # the reference arm runs once, on rank 0's GPU; the other ranks exit
        if rank != 0:
            return None
        world = 1
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(local)
    w = dict(WORKLOADS[args.workload])
    if args.threads:
        w["threads"] = args.threads
    if args.rounds and "rounds" in w:
        w["rounds"] = args.rounds
    if args.arena_gib:
        w["arena"] = int(args.arena_gib * GIB)
    if args.batches and "batches" in w:
        w["batches"] = args.batches
    if args.serve_slots and "slots" in w:
        w["slots"] = args.serve_slots
    if args.keys and "keys" in w:
        w["keys"] = args.keys
        w["buckets"] = max(args.keys // 4, 1)
    if args.vectors and "vectors" in w:
        w["vectors"] = args.vectors
    if args.drop_freed:
        w["drop_freed"] = True
    if args.batch_hi and "batches" in w:
        w["batch_hi"] = args.batch_hi
    if args.batch_form and "form" in w:
        w["form"] = args.batch_form
    impl = args.impl
    if impl == "reference":
        import oracle

        if args.workload == "mixed":
            # Not run again: on this workload the reference's CUDA build trapped
            # (cudaErrorLaunchFailure, Xid 43). A segment-tier free puts its
            # segments back in the segment tree before it resets their
            # memory-table tag (reference gallatin.cuh:1283-1302), so a
            # concurrent attach or gather finds the old tag in set_tree_id and
            # executes `trap` (gallatin.cuh:802-811, 1477-1489).
            if rank == 0:
                print(json.dumps({
                    "impl": "reference",
                    "unavailable": "the reference CUDA build trapped on this workload (segment-tier free returns "
                                   "segments before resetting their tag, gallatin.cuh:1283-1302; a concurrent attach "
                                   "traps in set_tree_id, gallatin.cuh:1477-1489); not run again",
                }))
            return None
        if args.workload == "calloc":
            if rank == 0:
                print(json.dumps({
                    "impl": "reference",
                    "unavailable": "the reference's running_calloc needs dynamic parallelism with relocatable device "
                                   "code (gallatin.cuh:1306-1369) and its block clear returns blocks without zeroing "
                                   "them (memory_table.cuh:101-136), so it is not a zeroed-memory allocator to "
                                   "compare with",
                }))
            return None
        if oracle.load_ref() is None:
            if rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": "reference CUDA build (oracle/_ref) is not built"}))
            return None
    else:
        import gallatin_gb300 as gal

        gal.load()

    serving = args.workload in ("serving", "serving-spill")
    unit = {"batches": "requests/s", "serving": "pages/s", "serving-spill": "pages/s", "table": "key ops/s",
            "vectors": "pushes/s"}.get(
        args.workload, "malloc+free pairs/s")
    stream = torch.cuda.current_stream()
    s_ptr = stream.cuda_stream
    a = make_allocator(impl, w)
    ha = None
    if args.workload in ("spill", "serving-spill"):
        try:
            ha = make_allocator(impl, w, host=True)
        except RuntimeError as e:
            close_allocator(impl, a)
            if rank == 0:
                print(json.dumps({"impl": impl, "unavailable": f"host-arena allocator: {e}"}))
            return None
    launches_per_step = 1
    stats = torch.zeros(8, dtype=torch.int64, device="cuda")
    flush = torch.empty(256 * MIB, dtype=torch.uint8, device="cuda")

    if args.workload == "spill":
        from gallatin_gb300.workload import mixed_class_trace

        n = w["threads"]
        trace = mixed_class_trace(n, 1, 42).reshape(-1)
        d_trace = torch.from_numpy(trace).cuda()
        h_trace = torch.from_numpy(trace).pin_memory()
        d_table = torch.zeros(n, dtype=torch.int64, device="cuda")
        units = n
        # 8 B pointer record written and read back, 16 B payload written and
        # 16 B read back per allocation
        alg_bytes = n * 48
        launches_per_step = 2

        def step():
            a.run_fused(ha, n, 42, d_table.data_ptr(), stats.data_ptr(), d_classes=d_trace.data_ptr(), phases=3,
                        stream=s_ptr)

        e2e_step = None
        if impl == "gb300":
            def e2e_step():
                return a.run_fused_host(ha, n, 42, h_trace.data_ptr(), stream=s_ptr)

        h2d = n
        config = {
            "workload": "device-first malloc with a pinned host-arena fallback (fused): fill n allocations of "
                        "16..4096 B powers of two, then verify and free each",
            "arena_bytes": w["arena"], "host_arena_bytes": w["host_arena"], "segment_bytes": w["segment"],
            "min_size": w["min_size"], "max_size": w["max_size"], "allocations": n, "seed": 42,
            "l2": "flushed (256 MiB write) before every timed step",
        }
    elif args.workload in ("mixed", "mixed-slices", "calloc"):
        from gallatin_gb300.workload import mixed_class_trace, mixed_mean_bytes

        n, rounds = w["threads"], w["rounds"]
        trace = mixed_class_trace(n, rounds, 42)
        d_trace = torch.from_numpy(trace.reshape(-1)).cuda()
        h_trace = torch.from_numpy(trace.reshape(-1)).pin_memory()
        seg_requests = n // w["block"] // w["seg_every"] if w["seg_every"] else 0
        units = n * rounds + seg_requests
        alg_bytes = n * rounds * 2 * mixed_mean_bytes() + seg_requests * 64

        def step():
            a.run_mixed(n, rounds, 42, stats.data_ptr(), seg_every=w["seg_every"], seg_lo=w["seg_lo"],
                        seg_hi=w["seg_hi"], d_classes=d_trace.data_ptr(), block_dim=w["block"], stream=s_ptr)

        def e2e_step():
            return a.run_mixed_host(n, rounds, 42, h_trace.data_ptr(), seg_every=w["seg_every"],
                                    seg_lo=w["seg_lo"], seg_hi=w["seg_hi"], block_dim=w["block"], stream=s_ptr)

        h2d = n * rounds
        if args.workload == "calloc":
            alg_bytes += n * rounds * mixed_mean_bytes()  # the zeroing write of every free
        config = {
            "workload": "mixed sizes 16..4096 B powers of two, 8 rounds malloc/fill/verify/free" + (
                ", zeroed on free (calloc)" if args.workload == "calloc" else ""),
            "arena_bytes": w["arena"], "segment_bytes": w["segment"], "min_size": w["min_size"],
            "max_size": w["max_size"], "threads": n, "rounds": rounds, "block_dim": w["block"],
            "segment_tier_requests": seg_requests, "segment_tier_bytes": [w["seg_lo"], w["seg_hi"]], "seed": 42,
            "l2": "flushed (256 MiB write) before every timed step",
        }
    elif args.workload == "batches":
        from gallatin_gb300.workload import batch_trace, prefix_with_drain

        reqs, offsets, slots, info = batch_trace(42, n_batches=w["batches"], batch_hi=w.get("batch_hi", 524288))
        sample = None
        if impl == "reference":
            # The reference's plain path runs this stream's first batches at
            # full speed, but from batch 45 its mallocs return NULL (blocks are
            # recycled only once all 4096 slices are back) and a batch takes a
            # minute; its arm is timed on the first 40 batches plus a drain.
            reqs, offsets = prefix_with_drain(reqs, offsets, REF_BATCH_PREFIX)
            sample = f"first {REF_BATCH_PREFIX} of {w['batches']} batches, then a drain batch"
        units = int(offsets[-1])
        alg_bytes = units * 8  # the live-set table entry each request writes
        d_reqs = torch.from_numpy(reqs.view(np.int64)).cuda()
        d_offs = torch.from_numpy(offsets.view(np.int64)).cuda()
        d_table = torch.zeros(slots + 1, dtype=torch.int64, device="cuda")
        h_reqs = torch.from_numpy(reqs.view(np.int64)).pin_memory()
        bargs = (d_reqs.data_ptr(), d_offs.data_ptr(), offsets, d_table.data_ptr(), stats.data_ptr())
        if impl == "reference":
            def step():
                a.run_batches(*bargs, persistent=False, stream=s_ptr)

            e2e_step = None
            launches_per_step = int(np.count_nonzero(np.diff(offsets)))  # one per non-empty batch
        else:
            graph = a.capture_batches(*bargs, width=w["width"], **batch_form(w["form"]))
            if w["form"] == "launches":
                launches_per_step = int(np.count_nonzero(np.diff(offsets)))  # one per non-empty batch

            def step():
                graph.launch(s_ptr)

            def e2e_step():
                return a.run_batches_host(reqs, offsets, slots, width=w["width"], **batch_form(w["form"]),
                                          stream=s_ptr, reqs_ptr=h_reqs.data_ptr())

        h2d = units * 8 + len(offsets) * 8
        config = {
            "workload": f"batching: {w['batches']} batches of U[1k,{w.get('batch_hi', 524288) // 1024}k] requests, "
                        "lognormal(ln 256, 1.5) sizes in [16 B, 64 MiB], "
                        "60/40 malloc/free over the live set, then a drain batch",
            "arena_bytes": w["arena"], "segment_bytes": w["segment"], "min_size": w["min_size"],
            "max_size": w["max_size"], "requests": units, "mallocs": info["mallocs"], "frees": info["frees"],
            "max_live": info["max_live"], "max_request_bytes": info["max_request_bytes"], "seed": 42,
            "path": ("reference: one launch per batch" if impl == "reference"
                     else BATCH_FORM_TEXT[w["form"]] + f", captured once in a CUDA graph, aggregation width {w['width']}"),
            "l2": "flushed (256 MiB write) before every timed step",
        }
        if sample:
            config["sample"] = sample
            config["requests"] = units
    elif args.workload == "table":
        from gallatin_gb300.workload import splitmix64

        n, nb = w["keys"], w["buckets"]
        units = n * 2  # n inserts, n/2 erases, n/2 reinserts
        alg_bytes = units * 16  # a key and its value per op
        ops = ["insert", "erase_half", "compact", "reinsert_half", "clear"]
        if impl == "reference":
            heads = torch.zeros(nb, dtype=torch.int64, device="cuda")
            from gallatin_gb300 import TABLE_OPS

            def run_ops(names, d_keys=None, st=stats):
                for op in names:
                    a.table_op(heads.data_ptr(), nb, 9, TABLE_OPS[op], n, st.data_ptr(), d_keys=d_keys,
                               stream=s_ptr)
        else:
            tbl = a.table(nb, seed=9)

            def run_ops(names, d_keys=None, st=stats):
                for op in names:
                    tbl.op(op, n, st.data_ptr(), d_keys=d_keys, stream=s_ptr)

        def step():
            run_ops(ops)

        launches_per_step = len(ops)  # one kernel per table operation

        with np.errstate(over="ignore"):
            h_keys = torch.from_numpy(splitmix64(np.arange(n, dtype=np.uint64) + np.uint64(42)).view(np.int64))
        h_keys = h_keys.pin_memory()
        d_keys_buf = torch.empty(n, dtype=torch.int64, device="cuda")
        e2e_stats = torch.zeros(8, dtype=torch.int64, device="cuda")
        h_stats = torch.zeros(8, dtype=torch.int64).pin_memory()

        def e2e_step():
            e2e_stats.zero_()
            d_keys_buf.copy_(h_keys, non_blocking=True)
            run_ops(ops, d_keys=d_keys_buf.data_ptr(), st=e2e_stats)
            h_stats.copy_(e2e_stats, non_blocking=True)
            torch.cuda.synchronize()
            out = np.zeros(8, dtype=np.uint64)
            out[0] = h_stats[0].item() + h_stats[1].item()
            return out

        h2d = n * 8
        config = {
            "workload": f"chained hash table: {n} uniform u64 keys (splitmix64 from seed 42), insert all, erase a "
                        "random half, compact empty nodes, reinsert the half, free all; 120 B nodes",
            "arena_bytes": w["arena"], "segment_bytes": w["segment"], "min_size": w["min_size"],
            "max_size": w["max_size"], "keys": n, "buckets": nb, "seed": 42,
            "path": "one thread per key, nodes from the allocator under test",
            "l2": "flushed (256 MiB write) before every timed step; table state exceeds L2",
        }
    elif args.workload == "vectors":
        from gallatin_gb300.workload import vector_lengths

        lengths = vector_lengths(w["vectors"])
        units = int(lengths.sum())
        alg_bytes = units * 8  # 4 B per push plus about 4 B copied per push over the doublings
        d_len = torch.from_numpy(lengths.view(np.int32)).cuda()
        h_len = torch.from_numpy(lengths.view(np.int32)).pin_memory()
        d_len_e2e = torch.empty_like(d_len)

        def step():
            a.run_vectors(d_len.data_ptr(), len(lengths), stats.data_ptr(), stream=s_ptr)

        e2e_stats = torch.zeros(8, dtype=torch.int64, device="cuda")
        h_stats = torch.zeros(8, dtype=torch.int64).pin_memory()

        def e2e_step():
            e2e_stats.zero_()
            d_len_e2e.copy_(h_len, non_blocking=True)
            a.run_vectors(d_len_e2e.data_ptr(), len(lengths), e2e_stats.data_ptr(), stream=s_ptr)
            h_stats.copy_(e2e_stats, non_blocking=True)
            torch.cuda.synchronize()
            out = np.zeros(8, dtype=np.uint64)
            out[0] = h_stats[0].item()
            out[1] = h_stats[2].item()
            return out

        h2d = len(lengths) * 4
        config = {
            "workload": f"{len(lengths)} per-thread u32 vectors grown by push_back to lognormal(ln 64, 1.5) "
                        "lengths capped at 65,536, doubling by malloc/copy/free, then checked and freed",
            "arena_bytes": w["arena"], "segment_bytes": w["segment"], "min_size": w["min_size"],
            "max_size": w["max_size"], "vectors": len(lengths), "pushes": units, "seed": 42,
            "l2": "flushed (256 MiB write) before every timed step",
        }
    elif serving:
        from gallatin_gb300.serving import ServingRun
        from gallatin_gb300.workload import serving_trace

        if args.serve_steps:
            w["steps"] = args.serve_steps
        elif impl == "reference":
            w["steps"] = REF_SERVE_STEPS
        trace = serving_trace(42, steps=w["steps"], arrivals_per_step=w["arrivals"])
        budget = int(w["gate"] * (w["arena"] + w.get("host_arena", 0))) // w["page_bytes"]
        if ha is not None:
            # device first, the host arena when the device has no page
            def entry(*x):
                return a.run_serving_fused(ha, *x)
        else:
            entry = a.run_serving
        srv_kw = dict(budget_pages=budget, page_bytes=w["page_bytes"], max_slots=w["slots"], max_pages=w["max_pages"])
        srv = ServingRun(torch, trace, **srv_kw)
        persistent = impl != "reference"

        geo = w["ctas_per_sm"] if persistent else 0
        # the loop's own kernels per run: two init kernels, then one
        # cooperative launch (device loop) or a prologue, two per step and a
        # drain (plain path)
        launches_per_step = 3 if persistent else 2 + 1 + 2 * w["steps"] + 1

        def step():
            srv.run(entry, persistent=persistent, ctas_per_sm=geo, stream=s_ptr)

        def e2e_step():
            r = ServingRun(torch, trace, **srv_kw)  # trace to the device
            r.run(entry, persistent=persistent, ctas_per_sm=geo, stream=s_ptr)
            res_e = r.results()  # outputs back to the host
            out = np.zeros(8, dtype=np.uint64)
            out[0] = res_e["step_stats"][:, 7].sum()
            return out

        n_str = len(trace["pages"])
        h2d = (w["steps"] + 1) * 4 + n_str * 8 + (n_str + 1) * 8
        d2h = n_str * 16 + w["steps"] * 80 + 864 * 8
        units = None  # pages of one run, read back after the warm-up
        config = {
            "workload": f"serving: Poisson arrivals 2,000 streams/s, 0.5 s per step, {w['steps']} steps, "
                        "lognormal(ln 1024, 1.0) tokens in [128, 32768], one 8 KiB page (16 tokens) per step per "
                        "stream, pages freed at completion, admission gated at 80 % of the arena" + (
                            "s (device and pinned host); pages device-first, host arena on NULL" if ha is not None
                            else ""),
            "arena_bytes": w["arena"], "host_arena_bytes": w.get("host_arena", 0), "segment_bytes": w["segment"],
            "min_size": w["min_size"],
            "max_size": w["max_size"], "steps": w["steps"], "streams": n_str, "budget_pages": budget,
            "slots": w["slots"], "seed": 42,
            "path": ("reference: plain path, one launch per phase per step" if impl == "reference"
                     else f"device-resident loop: one cooperative launch for all steps, {w['ctas_per_sm']} CTA/SM"),
            "l2": "flushed (256 MiB write) before every timed step",
        }
    else:
        n = w["threads"]
        units = n
        alg_bytes = n * 16

        def step():
            a.run_pairs(n, w["size"], stats.data_ptr(), block_dim=w["block"], stream=s_ptr)

        e2e_step = None
        h2d = 0
        config = {
            "workload": "plain 16 B malloc/store/verify/free", "arena_bytes": w["arena"], "segment_bytes": w["segment"],
            "min_size": w["min_size"], "max_size": w["max_size"], "threads": n, "block_dim": w["block"], "seed": 42,
            "l2": "flushed (256 MiB write) before every timed step",
        }

    # the per-thread workloads of our allocator run their whole timed loop in
    # the library's native driver (gal_bench): warm-up, L2 flush, CUDA events,
    # and the end-to-end leg through the host-buffer entry point
    native = None
    if impl == "gb300" and args.workload in ("mixed", "mixed-slices", "calloc", "pairs"):
        if args.workload == "pairs":
            native = dict(workload="pairs", n_threads=w["threads"], size=w["size"], block_dim=w["block"])
        else:
            native = dict(workload="mixed", n_threads=w["threads"], rounds=w["rounds"], seed=42,
                          seg_every=w["seg_every"], seg_lo=w["seg_lo"], seg_hi=w["seg_hi"],
                          d_classes=d_trace.data_ptr(), block_dim=w["block"])
            if not args.no_e2e:
                native["h_classes"] = h_trace.data_ptr()
        config["driver"] = "native (gal_bench: CUDA events on the launching stream)"
    if impl == "gb300" and w.get("drop_freed"):
        config["freed_lines"] = "GAL_FLAG_DROP_FREED: free drops freed 128 B-4 KiB slices' L2 lines without write-back"

    if native is None:
        for _ in range(args.warmup):
            step()
    torch.cuda.synchronize()
    stats.zero_()
    if serving:
        units = int(srv.results()["step_stats"][:, 0].sum())
        alg_bytes = units * 256  # 16 tokens written into each page and read back

    times = []
    native_out = None
    barrier(torch, world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        if native is not None:
            native_out = a.bench(**native, steps=args.steps, warmup=args.warmup, flush_bytes=flush.numel(),
                                 stream=s_ptr)
            times = native_out["step_ms"]
        else:
            for _ in range(args.steps):
                flush.fill_(1)
                ev0 = torch.cuda.Event(enable_timing=True)
                ev1 = torch.cuda.Event(enable_timing=True)
                ev0.record(stream)
                step()
                ev1.record(stream)
                ev1.synchronize()
                times.append(ev0.elapsed_time(ev1))
        torch.cuda.synchronize()
    barrier(torch, world)
    st = native_out["stats"] if native_out is not None else stats.cpu().numpy()
    total_ms = barrier_max(torch, world, float(sum(times)))
    ms_per_step = total_ms / args.steps
    value = replica_throughput(units, args.steps, world, total_ms)

    e2e = None
    if native_out is not None and native_out["e2e_step_ms"] is not None:
        e2e_total = barrier_max(torch, world, float(sum(native_out["e2e_step_ms"])) / 1e3)
        e2e = {
            "value": replica_throughput(units, args.steps, world, e2e_total * 1e3),
            "unit": unit,
            "h2d_bytes_per_step": h2d,
            "d2h_bytes_per_step": 64,
            "ms_per_step": 1e3 * e2e_total / args.steps,
            "misses": int(native_out["e2e_stats"][0]),
            "verify_failures": int(native_out["e2e_stats"][1]),
        }
    elif e2e_step is not None and not args.no_e2e and native is None:
        e2e_step()  # grow scratch buffers outside the timed region
        torch.cuda.synchronize()
        e2e_times = []
        e2e_bad = np.zeros(8, dtype=np.uint64)
        barrier(torch, world)
        for _ in range(args.steps):
            flush.fill_(1)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            out = e2e_step()
            e2e_times.append(time.perf_counter() - t0)
            e2e_bad += out
        e2e_total = barrier_max(torch, world, float(sum(e2e_times)))
        e2e = {
            "value": replica_throughput(units, args.steps, world, e2e_total * 1e3),
            "unit": unit,
            "h2d_bytes_per_step": h2d,
            "d2h_bytes_per_step": d2h if serving else 64,
            "ms_per_step": 1e3 * e2e_total / args.steps,
            "misses": int(e2e_bad[0]),
            "verify_failures": int(e2e_bad[1]),
        }

    peaks = measured_peaks()
    peak = peaks.get("hbm_gbs")
    achieved = alg_bytes / (ms_per_step / 1e3) / 1e9
    roofline = {
        "bound": "hbm",
        "achieved": achieved,
        "peak": peak if peak else 6800.0,
        "unit": "GB/s",
        "frac": achieved / (peak if peak else 6800.0),
        "traffic": None,
        "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if peak else "fallback 6.8 TB/s",
        "algorithmic_bytes_per_launch": alg_bytes,
    }
    traffic_file = REPO / "profiles" / f"traffic_{impl}_{args.workload}.json"
    traffic = {}
    if traffic_file.exists():
        try:
            traffic = json.loads(traffic_file.read_text())
        except ValueError:
            traffic = {}
        roofline["traffic"] = traffic.get("dram_bytes_per_launch")
    if roofline["traffic"]:
        # DRAM-side fraction: the bytes the dominant kernel really moved per
        # launch (ncu) over the same device time
        dram_gbs = roofline["traffic"] / (ms_per_step / 1e3) / 1e9
        roofline["dram"] = {"achieved": dram_gbs, "frac": dram_gbs / roofline["peak"]}
    if impl == "gb300":
        # the allocator's own roofline: L2 atomics per second against the
        # probe's peak, atomics per unit from an ncu count of the same kernel
        roofline["l2_atomic"] = l2_atomic_roofline(torch, stream, traffic.get("l2_atomics_per_unit"),
                                                   units / (ms_per_step / 1e3))

    result = {
        "metric": {"batches": "malloc+free ops/s (one op = one malloc or one free request)",
                   "serving": "page allocations/s of the serving loop (p50/p99 page-malloc latency in 'serving')",
                   "serving-spill": "page allocations/s of the serving loop over device + host arenas (p50/p99 "
                                    "page-malloc latency in 'serving')",
                   "table": "chained hash table key ops/s (insert + erase + reinsert, nodes from the allocator)",
                   "vectors": "vector push_back/s (doubling backings from the allocator)",
                   }.get(args.workload, "malloc+free ops/s (one op = one malloc + its free)"),
        "value": value,
        "unit": unit,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_per_step,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u64",
        "data": "synthetic (seeded xorshift64 size trace; no dataset)",
        "config": config,
        "impl": impl,
        "roofline": roofline,
        "e2e": e2e,
        "clocks": clocks.summary(),
        "gpu_launches": args.steps * launches_per_step,
        "misses": int(st[0]),
        "verify_failures": int(st[1]),
        "step_ms": times,
    }
    if args.workload in ("mixed", "mixed-slices", "calloc"):
        # stats words 2 and 3 of the mixed kernel: segment-tier requests served / NULL
        result["segment_tier"] = {"ok": int(st[2]), "null": int(st[3])}
    elif args.workload == "table":
        # stats word 3 of the table kernel: nodes freed (compaction and clear) over the timed steps
        result["nodes_freed"] = int(st[3])
    if args.workload == "table":
        # untimed check of the whole lifecycle: every key where it should be
        chk = torch.zeros(8, dtype=torch.int64, device="cuda")
        run_ops(["insert", "erase_half", "query_after_erase", "compact", "reinsert_half", "query", "clear"], st=chk)
        c = chk.cpu().numpy()
        result["checks"] = {"insert_failures": int(c[0]), "membership_errors": int(c[1]), "wrong_values": int(c[2])}
        result["verify_failures"] = int(c[1] + c[2])
        if impl == "gb300":
            tbl.close()
    if args.workload == "vectors":
        result["verify_failures"] = int(st[2])
        result["checks"] = {"pushes": int(st[4]), "expected_pushes": units * args.steps}
    if serving:
        from gallatin_gb300.serving import summarize
        from gallatin_gb300.workload import serving_admission

        res = srv.results()
        result["serving"] = summarize(res, page_bytes=w["page_bytes"], segment_bytes=w["segment"],
                                      seconds=ms_per_step / 1e3)
        admit_model, _ = serving_admission(trace, budget, w["slots"])
        result["serving"]["admission_matches_model"] = bool(np.array_equal(res["admit_step"], admit_model))
        if impl == "gb300" and not args.no_prefix and ha is None:
            # the plain path (one launch per phase per step) on the same trace
            srv0 = ServingRun(torch, trace, **srv_kw)
            srv0.run(a.run_serving, persistent=False, stream=s_ptr)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            flush.fill_(1)
            e0.record(stream)
            srv0.run(a.run_serving, persistent=False, stream=s_ptr)
            e1.record(stream)
            e1.synchronize()
            ms0 = e0.elapsed_time(e1)
            res0 = srv0.results()
            plain = summarize(res0, page_bytes=w["page_bytes"], segment_bytes=w["segment"], seconds=ms0 / 1e3)
            plain["ms_per_run"] = ms0
            plain["same_results"] = bool(np.array_equal(res0["checksum"], res["checksum"]) and
                                         np.array_equal(res0["admit_step"], res["admit_step"]))
            result["serving"]["plain_path"] = plain
        if impl == "gb300" and not args.no_prefix:
            # the device loop on the reference arm's sample (its first steps)
            if w["steps"] != REF_SERVE_STEPS:
                tr_s = serving_trace(42, steps=REF_SERVE_STEPS, arrivals_per_step=w["arrivals"])
                srv_s = ServingRun(torch, tr_s, **srv_kw)
                srv_s.run(entry, persistent=True, ctas_per_sm=geo, stream=s_ptr)
                torch.cuda.synchronize()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                flush.fill_(1)
                e0.record(stream)
                srv_s.run(entry, persistent=True, ctas_per_sm=geo, stream=s_ptr)
                e1.record(stream)
                e1.synchronize()
                ms_s = e0.elapsed_time(e1)
                short = summarize(srv_s.results(), page_bytes=w["page_bytes"], segment_bytes=w["segment"],
                                  seconds=ms_s / 1e3)
                short["ms_per_run"] = ms_s
                short["sample"] = f"first {REF_SERVE_STEPS} steps (the reference arm's sample)"
                result["serving"]["reference_sample"] = short
    if args.workload == "batches" and impl == "gb300":
        graph.close()
        if not args.no_prefix:
            result["prefix"] = batch_prefix_rates(torch, a, reqs, offsets, slots, w, stats, flush, args.steps)
        if args.autotune:
            from gallatin_gb300.autotune import autotune_batches

            close_allocator(impl, a)
            a = None
            result_autotune = autotune_batches(reqs, offsets, slots, arena=w["arena"])
    if args.workload == "spill":
        result["spill"] = {"host_served": int(st[4]), "host_fraction": int(st[4]) / max(units * args.steps, 1)}
    if ha is not None:
        close_allocator(impl, ha)
    if impl == "gb300" and a is not None and args.workload in ("mixed", "mixed-slices", "calloc"):
        # untimed end-state check of the whole run (timed and e2e steps): with
        # every allocation freed and the pinned blocks flushed, every tree and
        # table must equal its state after creation
        a.flush_pinned(s_ptr)
        torch.cuda.synchronize()
        rep = a.check_restored()
        result["checks"] = {"restored": rep["restored"],
                            "differences": {k: v for k, v in rep.items() if k != "restored" and v}}
    if impl == "gb300" and a is not None:
        st_all = a.stats()
        result["allocator_counters"] = st_all["counters"]
        result["tree_pins"] = st_all["tree_pins"]
    if a is not None:
        close_allocator(impl, a)
    if args.workload == "batches" and impl == "gb300" and args.autotune:
        result["autotune"] = result_autotune
    if rank == 0 and impl == "gb300" and not args.no_cpu_baseline:
        result["cpu_baseline"] = cpu_baseline(args.workload, w)
        if serving:
            # the glibc replay computes every finished stream's checksum on the
            # host: the device must report the same ones
            want = result["cpu_baseline"].pop("_checksums")
            fin = res["finish_step"] != 0xFFFFFFFF
            result["serving"]["checksum_mismatches_vs_host_replay"] = int((res["checksum"][fin] != want[fin]).sum())
    if impl == "reference":
        result["cpu_baseline"] = {
            "value": value, "unit": unit, "cores": 0, "kind": "reference",
            "sample": "the reference's own CUDA build on this GPU (it has no CPU path), full workload",
        }
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    return result if rank == 0 else None


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="mixed")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--drop-freed", action="store_true",
                    help="create our allocator with GAL_FLAG_DROP_FREED: free drops freed slices' L2 lines")
    ap.add_argument("--threads", type=int, default=0, help="override the thread count (small profiling cases)")
    ap.add_argument("--rounds", type=int, default=0, help="override the rounds of the mixed workload")
    ap.add_argument("--arena-gib", type=float, default=0.0, help="override the arena size")
    ap.add_argument("--autotune", action="store_true", help="batches workload: add the segment x width sweep")
    ap.add_argument("--batches", type=int, default=0, help="override the batch count (small profiling cases)")
    ap.add_argument("--batch-hi", type=int, default=0, help="override the largest batch size")
    ap.add_argument("--batch-form", choices=sorted(BATCH_FORM_TEXT), default=None,
                    help="batches workload: how the stream is served (default: the workload's form)")
    ap.add_argument("--no-prefix", action="store_true",
                    help="batches: skip the timing on the reference's sample; serving: skip the plain-path run")
    ap.add_argument("--serve-steps", type=int, default=0, help="override the serving workload's step count")
    ap.add_argument("--serve-slots", type=int, default=0, help="override the serving loop's stream slots")
    ap.add_argument("--keys", type=int, default=0, help="override the table workload's key count (buckets = keys / 4)")
    ap.add_argument("--vectors", type=int, default=0, help="override the vector count")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    res = run(args)
    if res is not None:
        print(json.dumps(res))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())

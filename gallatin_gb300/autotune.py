"""Autotuner for the batched request path.

Stage 1 sweeps the segment size {4, 16, 64} MiB, the warp-aggregation width
{8, 16, 32} and the kernel form (persistent cooperative kernel, with or
without per-batch binning by size class, or one launch per batch), each
captured as a CUDA graph and replayed. Stage 2 sweeps the kernel geometry
(CTAs of 256 threads per SM) at the best stage-1 point when that point is a
persistent form. The plain per-thread path (one launch per batch, no
graph) is timed beside each segment size. A configuration qualifies only if
none of its mallocs returned NULL; the best qualifying one is reported.

A 4 MiB segment can only hold a block of 1 KiB slices (segment >= max_size *
4096, the reference's static_assert gallatin.cuh:300), so it is paired with
max_size = 1024; the other segment sizes use 4096.

Device buffers come from torch (any CUDA buffer provider would do); the
allocator itself is the compiled C ABI.
"""
from __future__ import annotations

import numpy as np

from . import Gallatin

SEGMENTS = (4 << 20, 16 << 20, 64 << 20)
WIDTHS = (8, 16, 32)
FORMS = ("persistent", "binned", "launches")
GEOMETRIES = (1, 2, 3, 4)


def _time_ms(torch, fn, reps: int) -> float:
    times = []
    for _ in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    return float(np.median(times))


def _max_size(seg: int) -> int:
    return 4096 if seg >= (16 << 20) else 1024


def autotune_batches(reqs: np.ndarray, offsets: np.ndarray, table_slots: int, *, arena: int = 8 << 30,
                     segments=SEGMENTS, widths=WIDTHS, forms=FORMS, geometries=GEOMETRIES, reps: int = 3,
                     seed: int = 42) -> dict:
    import torch

    n_ops = int(offsets[-1])
    d_reqs = torch.from_numpy(reqs.view(np.int64)).cuda()
    d_offs = torch.from_numpy(np.asarray(offsets, dtype=np.uint64).view(np.int64)).cuda()
    d_table = torch.zeros(table_slots + 1, dtype=torch.int64, device="cuda")
    stats = torch.zeros(8, dtype=torch.int64, device="cuda")
    args = (d_reqs.data_ptr(), d_offs.data_ptr(), offsets, d_table.data_ptr(), stats.data_ptr())

    def graph_row(a, seg, form, width, geometry):
        try:
            g = a.capture_batches(*args, width=width, persistent=form != "launches", binned=form == "binned",
                                  ctas_per_sm=geometry)
        except RuntimeError as e:  # more CTAs per SM than fit
            return {"path": form + "+graph", "segment_bytes": seg, "width": width, "ctas_per_sm": geometry,
                    "error": str(e)}
        with g:
            for _ in range(2):
                g.launch()
            torch.cuda.synchronize()
            stats.zero_()
            ms = _time_ms(torch, g.launch, reps)
        return {"path": form + "+graph", "segment_bytes": seg, "max_size": _max_size(seg), "width": width,
                "ctas_per_sm": geometry, "ms": ms, "ops_per_s": n_ops / (ms / 1e3), "misses": int(stats[0].item())}

    rows = []
    for seg in segments:
        a = Gallatin.generate_on_device(arena, seed, print_info=False, segment_size=seg, max_size=_max_size(seg))
        try:
            for form in forms:
                for w in widths:
                    rows.append(graph_row(a, seg, form, w, 0))
            a.run_batches(*args, width=32, persistent=False)
            torch.cuda.synchronize()
            stats.zero_()
            ms = _time_ms(torch, lambda: a.run_batches(*args, width=32, persistent=False), reps)
            rows.append({"path": "per-thread launches", "segment_bytes": seg, "max_size": _max_size(seg),
                         "width": 32, "ctas_per_sm": None, "ms": ms, "ops_per_s": n_ops / (ms / 1e3),
                         "misses": int(stats[0].item())})
        finally:
            a.free_on_device()

    def qualified(rs):
        return [r for r in rs if r["path"] != "per-thread launches" and "ms" in r and r["misses"] == 0]

    best = max(qualified(rows) or [r for r in rows if "ms" in r], key=lambda r: r["ops_per_s"])
    seg, form, width = best["segment_bytes"], best["path"].split("+")[0], best["width"]
    if form != "launches":  # one launch per batch has no persistent grid to size
        a = Gallatin.generate_on_device(arena, seed, print_info=False, segment_size=seg, max_size=_max_size(seg))
        try:
            for geometry in geometries:
                rows.append(graph_row(a, seg, form, width, geometry))
        finally:
            a.free_on_device()
    best = max(qualified(rows) or [r for r in rows if "ms" in r], key=lambda r: r["ops_per_s"])
    plain = max((r for r in rows if r["path"] == "per-thread launches"), key=lambda r: r["ops_per_s"])
    return {"ops": n_ops, "best": best, "best_per_thread": plain, "results": rows}

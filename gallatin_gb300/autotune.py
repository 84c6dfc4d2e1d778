"""Autotuner for the batched request path.

Sweeps the segment size {4, 16, 64} MiB and the warp-aggregation width
{8, 16, 32} on a given request stream, each as a CUDA graph of the
persistent cooperative kernel, and reports the plain per-thread path (one
launch per batch, no graph) next to it. A 4 MiB segment can only hold a
block of 1 KiB slices (segment >= max_size * 4096, the reference's
static_assert gallatin.cuh:300), so it is paired with max_size = 1024; the
other segment sizes use 4096.

Device buffers come from torch (any CUDA buffer provider would do); the
allocator itself is the compiled C ABI.
"""
from __future__ import annotations

import numpy as np

from . import Gallatin

SEGMENTS = (4 << 20, 16 << 20, 64 << 20)
WIDTHS = (8, 16, 32)


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


def autotune_batches(reqs: np.ndarray, offsets: np.ndarray, table_slots: int, *, arena: int = 8 << 30,
                     segments=SEGMENTS, widths=WIDTHS, reps: int = 3, seed: int = 42) -> dict:
    import torch

    n_ops = int(offsets[-1])
    d_reqs = torch.from_numpy(reqs.view(np.int64)).cuda()
    d_offs = torch.from_numpy(np.asarray(offsets, dtype=np.uint64).view(np.int64)).cuda()
    d_table = torch.zeros(table_slots + 1, dtype=torch.int64, device="cuda")
    stats = torch.zeros(8, dtype=torch.int64, device="cuda")
    rows = []
    for seg in segments:
        max_size = 4096 if seg >= (16 << 20) else 1024
        a = Gallatin.generate_on_device(arena, seed, print_info=False, segment_size=seg, max_size=max_size)
        try:
            args = (d_reqs.data_ptr(), d_offs.data_ptr(), offsets, d_table.data_ptr(), stats.data_ptr())
            for w in widths:
                with a.capture_batches(*args, width=w, persistent=True) as g:
                    for _ in range(2):
                        g.launch()
                    torch.cuda.synchronize()
                    stats.zero_()
                    ms = _time_ms(torch, g.launch, reps)
                misses = int(stats[0].item())
                rows.append({"path": "persistent+graph", "segment_bytes": seg, "max_size": max_size, "width": w,
                             "ms": ms, "ops_per_s": n_ops / (ms / 1e3), "misses": misses})
            a.run_batches(*args, width=32, persistent=False)
            torch.cuda.synchronize()
            stats.zero_()
            ms = _time_ms(torch, lambda: a.run_batches(*args, width=32, persistent=False), reps)
            rows.append({"path": "per-thread launches", "segment_bytes": seg, "max_size": max_size, "width": 32,
                         "ms": ms, "ops_per_s": n_ops / (ms / 1e3), "misses": int(stats[0].item())})
        finally:
            a.free_on_device()
    tuned = [r for r in rows if r["path"] == "persistent+graph" and r["misses"] == 0]
    best = max(tuned or rows, key=lambda r: r["ops_per_s"])
    return {"ops": n_ops, "best": best, "results": rows}

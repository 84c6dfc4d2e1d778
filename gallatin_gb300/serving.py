"""Host side of the serving loop (gal_run_serving): the C structs, device
copies of a stream trace (torch buffers), and the summary of a run.

The loop itself is device code (gallatin_gb300/csrc/serving.cuh); this module
only moves the trace in and the results out, and turns the latency histogram
into quantiles. `run` takes the entry point as a callable so the same driver
serves any allocator that exposes the C signature.
"""
from __future__ import annotations

import ctypes
from ctypes import c_uint32, c_uint64, c_void_p

import numpy as np

HIST_BUCKETS = 864
STATS = 10
STAT_NAMES = ("allocated", "finished", "freed", "live", "committed", "queued", "owned_segments", "misses",
              "phase1_ns", "phase2_ns")
NOT_SET = 0xFFFFFFFF


class ServeTrace(ctypes.Structure):
    _fields_ = [
        ("n_streams", c_uint32),
        ("pad_", c_uint32),
        ("arrivals_end", c_void_p),
        ("tokens", c_void_p),
        ("pages", c_void_p),
        ("page_prefix", c_void_p),
        ("ids", c_void_p),
    ]


class ServeParams(ctypes.Structure):
    _fields_ = [
        ("steps", c_uint32),
        ("tokens_per_page", c_uint32),
        ("page_bytes", c_uint64),
        ("budget_pages", c_uint64),
        ("seed", c_uint64),
        ("max_slots", c_uint32),
        ("max_pages", c_uint32),
        ("width", c_uint32),
        ("mode", c_uint32),
        ("ctas_per_sm", c_uint32),
        ("pad_", c_uint32),
    ]


class ServeOut(ctypes.Structure):
    _fields_ = [
        ("checksum", c_void_p),
        ("admit_step", c_void_p),
        ("finish_step", c_void_p),
        ("step_stats", c_void_p),
        ("latency_hist", c_void_p),
    ]


def bucket_lower_ns():
    """Lower bound (ns) of each latency bucket, and the bucket widths."""
    lo = np.zeros(HIST_BUCKETS, dtype=np.float64)
    width = np.ones(HIST_BUCKETS, dtype=np.float64)
    lo[:32] = np.arange(32)
    for b in range(32, HIST_BUCKETS):
        e = (b - 32) // 32 + 5
        sub = (b - 32) % 32
        lo[b] = (32 + sub) << (e - 5)
        width[b] = 1 << (e - 5)
    return lo, width


def quantile_ns(hist: np.ndarray, q: float) -> float:
    """q-quantile of a latency histogram, at the midpoint of its bucket."""
    hist = np.asarray(hist, dtype=np.float64)
    total = hist.sum()
    if total == 0:
        return float("nan")
    cum = np.cumsum(hist)
    b = int(np.searchsorted(cum, q * total, side="left"))
    lo, width = bucket_lower_ns()
    return float(lo[b] + width[b] / 2)


class ServingRun:
    """Device copies of one trace and the output buffers of a run."""

    def __init__(self, torch, trace: dict, *, budget_pages: int, page_bytes: int = 8192, max_slots: int = 262144,
                 max_pages: int = 2048, seed: int = 42, width: int = 32):
        if int(trace["pages"].max(initial=0)) > max_pages:
            raise ValueError("a stream needs more pages than max_pages")
        self.torch = torch
        self.trace = trace
        self.steps = int(trace["steps"])
        self.n = len(trace["pages"])
        dev = "cuda"

        def up(a, dtype):
            return torch.from_numpy(np.ascontiguousarray(a).view(dtype)).to(dev)

        self.d_arrivals_end = up(trace["arrivals_end"].astype(np.uint32), np.int32)
        self.d_tokens = up(trace["tokens"].astype(np.uint32), np.int32)
        self.d_pages = up(trace["pages"].astype(np.uint32), np.int32)
        self.d_prefix = up(trace["page_prefix"].astype(np.uint64), np.int64)
        self.d_ids = up(trace["ids"].astype(np.uint32), np.int32) if "ids" in trace else None
        n1 = max(self.n, 1)
        self.d_checksum = torch.zeros(n1, dtype=torch.int64, device=dev)
        self.d_admit = torch.zeros(n1, dtype=torch.int32, device=dev)
        self.d_finish = torch.zeros(n1, dtype=torch.int32, device=dev)
        self.d_stats = torch.zeros(self.steps * STATS, dtype=torch.int64, device=dev)
        self.d_hist = torch.zeros(HIST_BUCKETS, dtype=torch.int64, device=dev)
        self.c_trace = ServeTrace(self.n, 0, self.d_arrivals_end.data_ptr(), self.d_tokens.data_ptr(),
                                  self.d_pages.data_ptr(), self.d_prefix.data_ptr(),
                                  self.d_ids.data_ptr() if self.d_ids is not None else None)
        self.c_out = ServeOut(self.d_checksum.data_ptr(), self.d_admit.data_ptr(), self.d_finish.data_ptr(),
                              self.d_stats.data_ptr(), self.d_hist.data_ptr())
        self.base = dict(steps=self.steps, tokens_per_page=int(trace["tokens_per_page"]), page_bytes=page_bytes,
                         budget_pages=budget_pages, seed=seed, max_slots=max_slots, max_pages=max_pages, width=width)

    def params(self, persistent: bool = True, ctas_per_sm: int = 0) -> ServeParams:
        b = self.base
        return ServeParams(b["steps"], b["tokens_per_page"], b["page_bytes"], b["budget_pages"], b["seed"],
                           b["max_slots"], b["max_pages"], b["width"], 1 if persistent else 0, ctas_per_sm, 0)

    def run(self, entry, *, persistent: bool = True, ctas_per_sm: int = 0, stream: int = 0) -> None:
        """entry(trace*, params*, out*, stream) -> status, e.g. a bound
        gal_run_serving."""
        p = self.params(persistent, ctas_per_sm)
        rc = entry(ctypes.byref(self.c_trace), ctypes.byref(p), ctypes.byref(self.c_out), stream)
        if rc != 0:
            raise RuntimeError(f"serving entry point failed ({rc})")

    def results(self) -> dict:
        self.torch.cuda.synchronize()
        return {
            "checksum": self.d_checksum.cpu().numpy().view(np.uint64)[: self.n],
            "admit_step": self.d_admit.cpu().numpy().view(np.uint32)[: self.n],
            "finish_step": self.d_finish.cpu().numpy().view(np.uint32)[: self.n],
            "step_stats": self.d_stats.cpu().numpy().view(np.uint64).reshape(self.steps, STATS),
            "hist": self.d_hist.cpu().numpy().view(np.uint64),
        }


def summarize(res: dict, *, page_bytes: int, segment_bytes: int, seconds: float | None = None) -> dict:
    """Pages, latency quantiles and fragmentation of one run. Fragmentation at
    a step is 1 - live bytes / bytes of the segments the allocator holds; it
    is reported at the step of peak live pages and as the mean over the steps
    past the first tenth (the ramp-up)."""
    st = res["step_stats"].astype(np.float64)
    hist = res["hist"]
    pages = float(st[:, 0].sum())
    out = {
        "pages_allocated": int(pages),
        "streams_finished": int(st[:, 1].sum()),
        "malloc_nulls": int(st[:, 7].sum()),
        "latency_ns": {"p50": quantile_ns(hist, 0.50), "p99": quantile_ns(hist, 0.99),
                       "max_bucket": quantile_ns(hist, 1.0), "samples": int(hist.sum())},
        "peak_live_pages": int(st[:, 3].max(initial=0)),
        "peak_committed_pages": int(st[:, 4].max(initial=0)),
        "final_queue": int(st[-1, 5]) if len(st) else 0,
        "step_us": {"phase1_mean": float(st[:, 8].mean() / 1e3) if len(st) else 0.0,
                    "phase2_mean": float(st[:-1, 9].mean() / 1e3) if len(st) > 1 else 0.0,
                    "phase1_max": float(st[:, 8].max(initial=0) / 1e3)},
    }
    owned = st[:, 6]
    if len(st) and owned.max() < 2**60:
        held = owned * segment_bytes
        live = st[:, 3] * page_bytes
        frag = np.where(held > 0, 1.0 - live / np.maximum(held, 1), 0.0)
        k = int(st[:, 3].argmax())
        start = len(st) // 10
        out["fragmentation"] = {"at_peak_live": float(frag[k]), "mean": float(frag[start:].mean()),
                                "owned_bytes_at_peak": int(held[k])}
    else:
        out["fragmentation"] = None
    if seconds:
        out["pages_per_s"] = pages / seconds
    return out

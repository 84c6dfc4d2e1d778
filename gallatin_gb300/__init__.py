"""GB300-native Gallatin device allocator: host-side Python mirror of the C ABI.

The allocator itself is CUDA code: device malloc/free are header-only
(include/gallatin/allocators/gallatin.cuh) and the host library
libgallatin_gb300.so (include/gallatin_gb300.h) builds, inspects and destroys
allocator state and runs batch kernels over it. This module binds that
library with ctypes and mirrors the reference's host interface
(gallatin::allocators::Gallatin<seg, min, max>::generate_on_device /
generate_on_device_host / free_on_device / print_info, and the global
allocator functions of global_allocator.cuh:41-216: init_global_allocator /
free_global_allocator / print_global_stats, their _host and _combined forms).

Device buffers are passed as integer device addresses and streams as integer
cudaStream_t handles, so any CUDA buffer provider works (the tests use torch).
There is no CPU fallback: without the compiled library every entry point
raises.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_char_p, c_int, c_int64, c_uint8, c_uint32, c_uint64, c_void_p
from pathlib import Path

import numpy as np

from . import _build

__all__ = [
    "GalError",
    "Gallatin",
    "VebTree",
    "load",
    "lib_path",
    "init_global_allocator",
    "free_global_allocator",
    "print_global_stats",
    "global_allocator",
    "init_global_allocator_host",
    "free_global_allocator_host",
    "print_global_stats_host",
    "global_host_allocator",
    "init_global_allocator_combined",
    "free_global_allocator_combined",
    "FLAG_HOST_ARENA",
    "FLAG_CALLOC",
    "OPS",
    "DUMP",
    "COUNTERS",
    "classify",
]

GAL_MAX_TREES = 24
GAL_NUM_COUNTERS = 64
GAL_EMPTY_BLOCK = 0xFFFFFFFF
GAL_FREE_SEGMENT = 0xFFFF
GAL_SEG_GATE = -(1 << 28)
NOALLOC_TRACE_MAX_BYTES = 2 << 20
FLAG_HOST_ARENA = 1  # arena in pinned host memory mapped into the GPU
FLAG_CALLOC = 2  # malloc returns zeroed bytes (zero on free)
FLAG_DROP_FREED = 4  # free drops freed 128 B..4 KiB slices' L2 lines without write-back (off by default)

OPS = {
    "insert": 0,
    "insert_force_update": 1,
    "remove": 2,
    "query": 3,
    "successor": 4,
    "successor_thorough": 5,
    "lock_offset": 6,
    "malloc_first": 7,
    "find_first_valid_index": 8,
    "find_random_valid_index": 9,
    "malloc": 10,
    "gather_multiple": 11,
    "return_multiple": 12,
    "report_fill": 13,
    "find_at_or_after": 14,
    "claim_first": 15,
}

DUMP = {
    "chunk_ids": (0, np.uint16),
    "seg_avail": (1, np.int32),
    "seg_block_bits": (2, np.uint64),
    "block_meta": (3, np.uint64),
    "block_bits": (4, np.uint64),
    "slots": (6, np.uint64),
    "counters": (7, np.uint64),
    "segment_tree": (8, np.uint64),
    "sub_tree": (9, np.uint64),
    "locks": (10, np.uint32),
    "adopt_tree": (11, np.uint64),
    "roomy_tree": (12, np.uint64),
}

COUNTERS = [
    "oom_slice",
    "oom_block",
    "oom_segment",
    "timeout",
    "bad_free",
    "corrupt",
    "block_pins",
    "segment_attach",
    "segment_retire",
    "block_retire",
    "replace_empty",
    "replace_full",
    "replace_frag",
    "claim_short",
    "stale_slot",
    "slot_busy",
    "replace_refill",
    "adopt",
    "adopt_roomy",
    "nomem",
]
TREE_PIN_COUNTER = 32


class GalError(RuntimeError):
    """A C-ABI call returned an error status."""


def _batch_mode(persistent: bool, binned: bool) -> int:
    if not persistent:
        if binned:
            raise ValueError("binned batches need the persistent path")
        return 0
    return 2 if binned else 1


class _Geometry(ctypes.Structure):
    _fields_ = [
        ("segment_bytes", c_uint64),
        ("min_size", c_uint64),
        ("max_size", c_uint64),
        ("num_segments", c_uint64),
        ("arena_bytes", c_uint64),
        ("num_trees", c_uint32),
        ("blocks_per_segment", c_uint32),
        ("num_sms", c_uint32),
        ("total_slots", c_uint32),
        ("slot_count", c_uint32 * GAL_MAX_TREES),
        ("num_classes", c_uint32),
        ("flags", c_uint32),
        ("arena_base", c_uint64),
    ]


class _Stats(ctypes.Structure):
    _fields_ = [
        ("num_segments", c_uint64),
        ("free_segments", c_uint64),
        ("tree_segments", c_uint64 * GAL_MAX_TREES),
        ("tree_blocks_out", c_uint64 * GAL_MAX_TREES),
        ("tree_live_slices", c_uint64 * GAL_MAX_TREES),
        ("segment_allocations", c_uint64),
        ("segments_in_allocations", c_uint64),
        ("counters", c_uint64 * GAL_NUM_COUNTERS),
    ]


class _RestoreReport(ctypes.Structure):
    _fields_ = [
        ("segment_tree_words", c_uint64),
        ("sub_tree_words", c_uint64),
        ("adopt_tree_words", c_uint64),
        ("tagged_segments", c_uint64),
        ("open_segments", c_uint64),
        ("blocks_out", c_uint64),
        ("live_blocks", c_uint64),
        ("taken_slices", c_uint64),
        ("pinned_slots", c_uint64),
        ("corrupt", c_uint64),
        ("bad_frees", c_uint64),
        ("locks", c_uint32),
        ("restored", c_uint32),
    ]


class _BenchArgs(ctypes.Structure):
    _fields_ = [
        ("workload", c_uint32),
        ("block_dim", c_uint32),
        ("n_threads", c_uint64),
        ("size", c_uint64),
        ("rounds", c_uint32),
        ("seg_every", c_uint32),
        ("seed", c_uint64),
        ("seg_lo", c_uint64),
        ("seg_hi", c_uint64),
        ("d_classes", c_void_p),
        ("h_classes", c_void_p),
        ("warmup", c_uint32),
        ("steps", c_uint32),
        ("flush_bytes", c_uint64),
        ("stream", c_void_p),
    ]


class _BenchResult(ctypes.Structure):
    _fields_ = [
        ("step_ms", ctypes.POINTER(ctypes.c_float)),
        ("e2e_step_ms", ctypes.POINTER(ctypes.c_float)),
        ("stats", c_uint64 * 8),
        ("e2e_stats", c_uint64 * 8),
    ]


BENCH_WORKLOADS = {"pairs": 0, "mixed": 1}

SIZE_INFO_DTYPE = np.dtype([("tier", "<u4"), ("tree", "<u4"), ("count", "<u8"), ("allocated", "<u8")])
TIERS = ("slice", "block", "segment")

VEB_OP_DTYPE = np.dtype([("code", "<u4"), ("tid", "<u4"), ("arg", "<u8"), ("arg2", "<u8")])

_LIB = None


def lib_path() -> Path:
    return _build.lib_path()


def load(path: str | Path | None = None):
    """Load the compiled C-ABI library (raises if it has not been built)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    import os

    p = Path(path or os.environ.get("GALLATIN_GB300_LIB") or lib_path())
    if not p.exists():
        raise GalError(f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = ctypes.CDLL(str(p))
    vp, u64, u32, i32 = c_void_p, c_uint64, c_uint32, c_int
    sigs = {
        "gal_create": (i32, [u64, u64, u64, u64, u64, u32, POINTER(vp)]),
        "gal_create_ex": (i32, [u64, u64, u64, u64, u64, u32, u32, POINTER(vp)]),
        "gal_destroy": (i32, [vp]),
        "gal_device_state": (vp, [vp]),
        "gal_from_device_state": (vp, [vp]),
        "gal_geometry": (i32, [vp, POINTER(_Geometry)]),
        "gal_stats": (i32, [vp, POINTER(_Stats)]),
        "gal_print_info": (i32, [vp]),
        "gal_reset_counters": (i32, [vp]),
        "gal_dump_bytes": (c_int64, [vp, i32, i32, i32]),
        "gal_dump": (i32, [vp, i32, i32, i32, vp, u64]),
        "gal_veb_layer_count": (i32, [vp, i32, i32]),
        "gal_malloc_batch": (i32, [vp, vp, u64, vp, vp]),
        "gal_free_batch": (i32, [vp, vp, u64, vp]),
        "gal_flush_pinned": (i32, [vp, vp]),
        "gal_size_classes": (i32, [vp, vp, u64, vp, vp]),
        "gal_check_restored": (i32, [vp, POINTER(_RestoreReport)]),
        "gal_set_wait_limit": (i32, [vp, u32]),
        "gal_set_locks": (i32, [vp, u32]),
        "gal_probe_l2_atomics": (i32, [vp, u64, u32, u32, u32, vp, POINTER(u64), vp]),
        "gal_bench": (i32, [vp, POINTER(_BenchArgs), POINTER(_BenchResult)]),
        "gal_run_pairs": (i32, [vp, u64, u64, u32, vp, vp]),
        "gal_run_mixed": (i32, [vp, u64, u32, u64, u32, u64, u64, vp, u32, vp, vp]),
        "gal_run_mixed_host": (i32, [vp, u64, u32, u64, u32, u64, u64, vp, u32, vp, vp]),
        "gal_run_mixed_host_noalloc": (i32, [vp, u64, u32, u64, u32, u64, u64, vp, u32, vp, vp]),
        "gal_run_fused": (i32, [vp, vp, u64, u64, vp, vp, u32, vp, vp]),
        "gal_run_fused_host": (i32, [vp, vp, u64, u64, vp, vp, vp]),
        "gal_run_zeroed": (i32, [vp, u64, u32, u64, u32, u64, u64, vp, vp]),
        "gal_run_batches": (i32, [vp, vp, vp, vp, u32, vp, u32, u32, u32, vp, vp]),
        "gal_capture_batches": (i32, [vp, vp, vp, vp, u32, vp, u32, u32, u32, vp, POINTER(vp)]),
        "gal_graph_launch": (i32, [vp, vp]),
        "gal_graph_destroy": (i32, [vp]),
        "gal_run_batches_host": (i32, [vp, vp, vp, u32, u64, u32, u32, u32, vp, vp]),
        "gal_run_serving": (i32, [vp, vp, vp, vp, vp]),
        "gal_run_serving_fused": (i32, [vp, vp, vp, vp, vp, vp]),
        "gal_table_create": (i32, [vp, u64, u64, POINTER(vp)]),
        "gal_table_op": (i32, [vp, u32, vp, u64, u64, vp, vp]),
        "gal_table_chain_stats": (i32, [vp, POINTER(u64), POINTER(u64)]),
        "gal_table_destroy": (i32, [vp]),
        "gal_run_vectors": (i32, [vp, vp, u64, u32, vp, vp]),
        "gal_veb_create": (i32, [u64, u64, POINTER(vp)]),
        "gal_veb_destroy": (i32, [vp]),
        "gal_veb_num_layers": (i32, [vp]),
        "gal_veb_layer_words": (u64, [vp, i32]),
        "gal_veb_dump": (i32, [vp, i32, vp]),
        "gal_veb_run_ops": (i32, [vp, vp, u64, vp, vp]),
        "gal_veb_load": (i32, [vp, vp, u64]),
        "gal_veb_find_batch": (i32, [vp, vp, u64, vp, u32, vp]),
        "gal_last_error": (c_char_p, []),
    }
    for name, (res, args) in sigs.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def _check(rc: int) -> None:
    if rc != 0:
        msg = load().gal_last_error().decode(errors="replace")
        raise GalError(f"gallatin_gb300 call failed ({rc}): {msg}")


def probe_l2_atomics(d_words: int, nbytes: int, iters: int, mode: int = 0, ctas_per_sm: int = 8,
                     d_sink: int = 0, stream: int = 0) -> int:
    """Launch the L2 atomic throughput probe (gal_probe_l2_atomics) over a
    device buffer of nbytes (its 128-byte lines, rounded down to a power of
    two, plus one u64 of it used as the sink); returns the atomics issued."""
    lines = 1 << ((nbytes // 128).bit_length() - 1)
    if d_sink == 0:
        lines //= 2  # keep the sink outside the probed lines
        d_sink = d_words + lines * 128
    ops = c_uint64(0)
    _check(load().gal_probe_l2_atomics(d_words, lines, iters, mode, ctas_per_sm, d_sink, ctypes.byref(ops), stream))
    return ops.value


def _ceil_log2(v: int) -> int:
    return (v - 1).bit_length() if v > 1 else 0


def classify(size: int, min_size: int = 16, max_size: int = 4096, segment_size: int = 16 << 20):
    """Tier of a request, as the device dispatch computes it.

    Returns (tier, tree, count_or_nseg) with tier in {"slice", "block",
    "segment"} (reference gallatin.cuh:1141-1147, 1196-1260)."""
    min_shift = min_size.bit_length() - 1
    max_shift = max_size.bit_length() - 1
    num_trees = max_shift - min_shift + 1
    block_shift_min = min_shift + 12
    if size < min_size:
        return ("slice", 0, 1)
    cl = _ceil_log2(size)
    tree = cl - min_shift
    if tree < num_trees:
        return ("slice", tree, 1)
    bt = cl - block_shift_min
    if bt < 0:
        return ("slice", num_trees - 1, 1 << (tree - (num_trees - 1)))
    if bt < num_trees:
        return ("block", bt, 1)
    return ("segment", 0, (size - 1) // segment_size + 1)


class Gallatin:
    """Host handle of one device allocator (reference Gallatin<seg, min, max>)."""

    def __init__(self, handle: int, segment_size: int, min_size: int, max_size: int):
        self._h = handle
        self.segment_size = segment_size
        self.min_size = min_size
        self.max_size = max_size
        g = _Geometry()
        _check(load().gal_geometry(self._h, ctypes.byref(g)))
        self.num_segments = g.num_segments
        self.arena_bytes = g.arena_bytes
        self.num_trees = g.num_trees
        self.blocks_per_segment = g.blocks_per_segment
        self.num_sms = g.num_sms
        self.total_slots = g.total_slots
        self.num_classes = g.num_classes
        self.slot_count = list(g.slot_count)[: g.num_classes]
        self.arena_base = g.arena_base
        self.flags = g.flags
        self.host_arena = bool(g.flags & FLAG_HOST_ARENA)
        self.calloc = bool(g.flags & FLAG_CALLOC)

    @classmethod
    def generate_on_device(
        cls,
        max_bytes: int,
        seed: int,
        print_info: bool = True,
        running_calloc: bool = False,
        *,
        segment_size: int = 16 << 20,
        min_size: int = 16,
        max_size: int = 4096,
        min_slots: int = 0,
        drop_freed: bool = False,
    ) -> "Gallatin":
        """running_calloc: every malloc returns zeroed bytes (zero on free).
        drop_freed: free drops the L2 lines of freed 128 B..4 KiB slices
        without writing them back (GAL_FLAG_DROP_FREED)."""
        flags = (FLAG_CALLOC if running_calloc else 0) | (FLAG_DROP_FREED if drop_freed else 0)
        return cls._generate(max_bytes, seed, print_info, flags, segment_size, min_size, max_size, min_slots)

    @classmethod
    def generate_on_device_host(
        cls,
        max_bytes: int,
        seed: int,
        print_info: bool = True,
        running_calloc: bool = False,
        *,
        segment_size: int = 16 << 20,
        min_size: int = 16,
        max_size: int = 4096,
        min_slots: int = 0,
    ) -> "Gallatin":
        """The allocator over pinned host memory mapped into the GPU
        (reference generate_on_device_host, gallatin.cuh:423-526): the arena
        is host memory, the metadata stays on the device."""
        flags = FLAG_HOST_ARENA | (FLAG_CALLOC if running_calloc else 0)
        return cls._generate(max_bytes, seed, print_info, flags, segment_size, min_size, max_size, min_slots)

    @classmethod
    def _generate(cls, max_bytes, seed, print_info, flags, segment_size, min_size, max_size, min_slots):
        h = c_void_p()
        _check(load().gal_create_ex(max_bytes, seed, segment_size, min_size, max_size, min_slots, flags,
                                    ctypes.byref(h)))
        obj = cls(h.value, segment_size, min_size, max_size)
        if print_info:
            where = "pinned host" if flags & FLAG_HOST_ARENA else "device"
            print(
                f"Booted Gallatin with {obj.num_trees} trees in range {min_size}-{max_size} and "
                f"{max_bytes / 2**30:f} GB of {where} memory {obj.num_segments} segments"
            )
        return obj

    def owns_allocation(self, ptr: int) -> bool:
        """Whether a pointer lies in this allocator's arena (reference
        owns_allocation, gallatin.cuh:2027, memory_table.cuh:1346)."""
        return 0 <= ptr - self.arena_base < self.arena_bytes

    def free_on_device(self) -> None:
        if self._h:
            _check(load().gal_destroy(self._h))
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.free_on_device()

    @property
    def handle(self) -> int:
        if not self._h:
            raise GalError("allocator already freed")
        return self._h

    @property
    def device_ptr(self) -> int:
        """Device pointer user kernels receive (what generate_on_device returns in C++)."""
        return load().gal_device_state(self.handle)

    # -- batch device entry points ------------------------------------------
    def malloc_batch(self, d_sizes: int, n: int, d_ptrs: int, stream: int = 0) -> None:
        _check(load().gal_malloc_batch(self.handle, d_sizes, n, d_ptrs, stream))

    def free_batch(self, d_ptrs: int, n: int, stream: int = 0) -> None:
        _check(load().gal_free_batch(self.handle, d_ptrs, n, stream))

    def flush_pinned(self, stream: int = 0) -> None:
        _check(load().gal_flush_pinned(self.handle, stream))

    def run_pairs(self, n_threads: int, size: int, d_stats: int, block_dim: int = 1024, stream: int = 0) -> None:
        _check(load().gal_run_pairs(self.handle, n_threads, size, block_dim, d_stats, stream))

    def run_mixed(
        self,
        n_threads: int,
        rounds: int,
        seed: int,
        d_stats: int,
        *,
        seg_every: int = 0,
        seg_lo: int = 16 << 20,
        seg_hi: int = 256 << 20,
        d_classes: int = 0,
        block_dim: int = 256,
        stream: int = 0,
    ) -> None:
        _check(
            load().gal_run_mixed(
                self.handle, n_threads, rounds, seed, seg_every, seg_lo, seg_hi, d_classes, block_dim, d_stats, stream
            )
        )

    def run_mixed_host(
        self,
        n_threads: int,
        rounds: int,
        seed: int,
        h_classes_ptr: int,
        *,
        seg_every: int = 0,
        seg_lo: int = 16 << 20,
        seg_hi: int = 256 << 20,
        block_dim: int = 256,
        stream: int = 0,
    ) -> np.ndarray:
        out = np.zeros(8, dtype=np.uint64)
        _check(
            load().gal_run_mixed_host(
                self.handle,
                n_threads,
                rounds,
                seed,
                seg_every,
                seg_lo,
                seg_hi,
                h_classes_ptr,
                block_dim,
                out.ctypes.data,
                stream,
            )
        )
        return out

    def run_mixed_host_noalloc(
        self,
        n_threads: int,
        rounds: int,
        seed: int,
        h_classes_ptr: int,
        *,
        seg_every: int = 0,
        seg_lo: int = 16 << 20,
        seg_hi: int = 256 << 20,
        block_dim: int = 256,
        stream: int = 0,
    ) -> np.ndarray:
        """run_mixed_host for callers that may not allocate device memory.

        The scratch is a fixed array inside the library (at most
        NOALLOC_TRACE_MAX_BYTES of trace); concurrent calls share it and race."""
        out = np.zeros(8, dtype=np.uint64)
        _check(
            load().gal_run_mixed_host_noalloc(
                self.handle,
                n_threads,
                rounds,
                seed,
                seg_every,
                seg_lo,
                seg_hi,
                h_classes_ptr,
                block_dim,
                out.ctypes.data,
                stream,
            )
        )
        return out

    # -- device first, host arena fallback ------------------------------------
    def run_fused(self, host: "Gallatin | None", n: int, seed: int, d_table: int, d_stats: int, *,
                  d_classes: int = 0, phases: int = 3, stream: int = 0) -> None:
        """Fill/drain of n allocations through the fused calls (see
        gal_run_fused): this allocator first, `host` when it returns NULL.
        phases: 1 fill, 2 drain, 3 both."""
        _check(load().gal_run_fused(self.handle, host.handle if host is not None else None, n, seed, d_classes,
                                    d_table, phases, d_stats, stream))

    def run_fused_host(self, host: "Gallatin | None", n: int, seed: int, h_classes_ptr: int,
                       stream: int = 0) -> np.ndarray:
        """Both phases end to end from a host class trace; returns the 8 stats words."""
        out = np.zeros(8, dtype=np.uint64)
        _check(load().gal_run_fused_host(self.handle, host.handle if host is not None else None, n, seed,
                                         h_classes_ptr, out.ctypes.data, stream))
        return out

    def run_zeroed(self, n_threads: int, rounds: int, seed: int, d_stats: int, *, big_every: int = 0,
                   big_lo: int = 64 << 10, big_hi: int = 1 << 20, stream: int = 0) -> None:
        """Zeroed-memory check (see gal_run_zeroed): stats[1] counts
        allocations that held a non-zero byte."""
        _check(load().gal_run_zeroed(self.handle, n_threads, rounds, seed, big_every, big_lo, big_hi, d_stats,
                                     stream))

    # -- batched request streams ---------------------------------------------
    def run_batches(self, d_reqs: int, d_offsets: int, offsets: np.ndarray, d_table: int, d_stats: int, *,
                    width: int = 32, persistent: bool = True, binned: bool = False, ctas_per_sm: int = 0,
                    stream: int = 0) -> None:
        """Serve a batched request stream (see gal_run_batches); `offsets` is
        the host copy of the batch offsets. persistent=False is the plain
        one-launch-per-batch path; binned sorts each batch by size class;
        ctas_per_sm sets the persistent grid (0 = as many as fit)."""
        offsets = np.ascontiguousarray(offsets, dtype=np.uint64)
        _check(load().gal_run_batches(self.handle, d_reqs, d_offsets, offsets.ctypes.data, len(offsets) - 1, d_table,
                                      width, _batch_mode(persistent, binned), ctas_per_sm, d_stats, stream))

    def capture_batches(self, d_reqs: int, d_offsets: int, offsets: np.ndarray, d_table: int, d_stats: int, *,
                        width: int = 32, persistent: bool = True, binned: bool = False,
                        ctas_per_sm: int = 0) -> "Graph":
        offsets = np.ascontiguousarray(offsets, dtype=np.uint64)
        g = c_void_p()
        _check(load().gal_capture_batches(self.handle, d_reqs, d_offsets, offsets.ctypes.data, len(offsets) - 1,
                                          d_table, width, _batch_mode(persistent, binned), ctas_per_sm, d_stats,
                                          ctypes.byref(g)))
        return Graph(g.value)

    def run_batches_host(self, reqs: np.ndarray, offsets: np.ndarray, table_slots: int, *, width: int = 32,
                         persistent: bool = True, binned: bool = False, ctas_per_sm: int = 0, stream: int = 0,
                         reqs_ptr: int | None = None) -> np.ndarray:
        """End to end from host buffers; returns the 8 stats words."""
        offsets = np.ascontiguousarray(offsets, dtype=np.uint64)
        out = np.zeros(8, dtype=np.uint64)
        ptr = reqs_ptr if reqs_ptr is not None else np.ascontiguousarray(reqs, dtype=np.uint64).ctypes.data
        _check(load().gal_run_batches_host(self.handle, ptr, offsets.ctypes.data, len(offsets) - 1, table_slots, width,
                                           _batch_mode(persistent, binned), ctas_per_sm, out.ctypes.data, stream))
        return out

    # -- serving loop ---------------------------------------------------------
    def run_serving(self, trace_ptr, params_ptr, out_ptr, stream: int = 0) -> int:
        """gal_run_serving on this allocator (pointers to the structs of
        gallatin_gb300.serving); returns 0 or raises GalError."""
        _check(load().gal_run_serving(self.handle, trace_ptr, params_ptr, out_ptr, stream))
        return 0

    def run_serving_fused(self, host: "Gallatin", trace_ptr, params_ptr, out_ptr, stream: int = 0) -> int:
        """gal_run_serving_fused: pages from this allocator first, from `host`
        (a host-arena allocator) when it has none."""
        _check(load().gal_run_serving_fused(self.handle, host.handle, trace_ptr, params_ptr, out_ptr, stream))
        return 0

    # -- data structures ------------------------------------------------------
    def table(self, nbuckets: int, seed: int = 42) -> "Table":
        """A chained hash table whose nodes come from this allocator."""
        h = c_void_p()
        _check(load().gal_table_create(self.handle, nbuckets, seed, ctypes.byref(h)))
        return Table(h.value, nbuckets)

    def run_vectors(self, d_lengths: int, n: int, d_stats: int, *, start: int = 1, stream: int = 0) -> None:
        """n per-thread doubling vectors grown to d_lengths[v] items (gal_run_vectors)."""
        _check(load().gal_run_vectors(self.handle, d_lengths, n, start, d_stats, stream))

    # -- inspection -----------------------------------------------------------
    def stats(self) -> dict:
        s = _Stats()
        _check(load().gal_stats(self.handle, ctypes.byref(s)))
        nt = self.num_trees
        return {
            "num_segments": s.num_segments,
            "free_segments": s.free_segments,
            "tree_segments": list(s.tree_segments)[:nt],
            "tree_blocks_out": list(s.tree_blocks_out)[:nt],
            "tree_live_slices": list(s.tree_live_slices)[:nt],
            "segment_allocations": s.segment_allocations,
            "segments_in_allocations": s.segments_in_allocations,
            "counters": dict(zip(COUNTERS, list(s.counters)[: len(COUNTERS)])),
            "tree_pins": list(s.counters)[TREE_PIN_COUNTER : TREE_PIN_COUNTER + nt],
        }

    def bench(self, workload: str, n_threads: int, *, steps: int, warmup: int, flush_bytes: int,
              block_dim: int = 256, size: int = 16, rounds: int = 1, seed: int = 42, seg_every: int = 0,
              seg_lo: int = 16 << 20, seg_hi: int = 256 << 20, d_classes: int = 0, h_classes: int = 0,
              stream: int = 0) -> dict:
        """The native benchmark driver (gal_bench): warm-up, L2 flush before
        every timed step, CUDA-event device times, and with h_classes (a pinned
        host trace) the same steps end to end with host-clock times."""
        args = _BenchArgs(BENCH_WORKLOADS[workload], block_dim, n_threads, size, rounds, seg_every, seed, seg_lo,
                          seg_hi, d_classes or None, h_classes or None, warmup, steps, flush_bytes, stream or None)
        step_ms = (ctypes.c_float * steps)()
        e2e_ms = (ctypes.c_float * steps)() if h_classes else None
        res = _BenchResult(step_ms, e2e_ms, (c_uint64 * 8)(), (c_uint64 * 8)())
        _check(load().gal_bench(self.handle, ctypes.byref(args), ctypes.byref(res)))
        return {
            "step_ms": list(step_ms),
            "e2e_step_ms": list(e2e_ms) if e2e_ms is not None else None,
            "stats": np.array(list(res.stats), dtype=np.uint64),
            "e2e_stats": np.array(list(res.e2e_stats), dtype=np.uint64),
        }

    def size_classes(self, d_sizes: int, n: int, d_out: int, stream: int = 0) -> None:
        """Device size classing of n request sizes into n SIZE_INFO_DTYPE
        records (gal_size_classes): tier, tree, slices or segments, and the
        allocated bytes (reference get_allocated_size)."""
        _check(load().gal_size_classes(self.handle, d_sizes, n, d_out, stream))

    def check_restored(self) -> dict:
        """Differences between the current state and the state after
        creation (gal_check_restored); "restored" is True when there are none.
        Call after every allocation is freed and flush_pinned has run."""
        r = _RestoreReport()
        _check(load().gal_check_restored(self.handle, ctypes.byref(r)))
        out = {name: int(getattr(r, name)) for name, _ in _RestoreReport._fields_}
        out["restored"] = bool(out["restored"])
        return out

    def set_wait_limit(self, lock_spins: int) -> None:
        """Tries of the segment-tier lock before a segment-tier malloc returns
        NULL and counts a timeout (gal_set_wait_limit)."""
        _check(load().gal_set_wait_limit(self.handle, lock_spins))

    def set_locks(self, locks: int) -> None:
        """Overwrite the lock word while no kernel runs (gal_set_locks): a
        bit set here is held by nobody, so waits on it run to their bound."""
        _check(load().gal_set_locks(self.handle, locks))

    def print_info(self) -> None:
        _check(load().gal_print_info(self.handle))

    def reset_counters(self) -> None:
        _check(load().gal_reset_counters(self.handle))

    def dump(self, name: str, tree: int = 0, layer: int = 0) -> np.ndarray:
        which, dtype = DUMP[name]
        nbytes = load().gal_dump_bytes(self.handle, which, tree, layer)
        if nbytes < 0:
            raise GalError(f"no dump target {name} tree={tree} layer={layer}")
        out = np.empty(nbytes // np.dtype(dtype).itemsize, dtype=dtype)
        _check(load().gal_dump(self.handle, which, tree, layer, out.ctypes.data, nbytes))
        return out

    def veb_layers(self, tree: int = -1, kind: str = "sub_tree") -> list[np.ndarray]:
        """All layers (top first) of the segment tree (tree=-1), of sub tree
        `tree` (kind "sub_tree"), or of slot class `tree`'s adoptable-block or
        roomy-block tree (kind "adopt_tree" or "roomy_tree")."""
        if tree < 0:
            kind = "segment_tree"
        which = DUMP[kind][0]
        n = load().gal_veb_layer_count(self.handle, which, max(tree, 0))
        return [self.dump(kind, max(tree, 0), i) for i in range(n)]


TABLE_OPS = {"insert": 0, "erase_half": 1, "reinsert_half": 2, "query": 3, "compact": 4, "clear": 5,
             "query_after_erase": 6}
DS_STATS = ("no_node", "membership", "wrong_value", "nodes_freed", "pushes")


class Table:
    """gal_table: a chained hash table over an allocator (gal_table_*)."""

    def __init__(self, handle: int, nbuckets: int):
        self._t = handle
        self.nbuckets = nbuckets

    def op(self, name: str, n: int, d_stats: int, *, d_keys: int | None = None, key_seed: int = 42,
           stream: int = 0) -> None:
        _check(load().gal_table_op(self._t, TABLE_OPS[name], d_keys, n, key_seed, d_stats, stream))

    def chain_stats(self) -> tuple[int, int]:
        """(longest chain, total nodes)."""
        mx, tot = c_uint64(0), c_uint64(0)
        _check(load().gal_table_chain_stats(self._t, ctypes.byref(mx), ctypes.byref(tot)))
        return mx.value, tot.value

    def close(self) -> None:
        if self._t:
            _check(load().gal_table_destroy(self._t))
            self._t = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Graph:
    """An instantiated CUDA graph owned by the library (gal_capture_batches)."""

    def __init__(self, handle: int):
        self._g = handle

    def launch(self, stream: int = 0) -> None:
        _check(load().gal_graph_launch(self._g, stream))

    def close(self) -> None:
        if self._g:
            _check(load().gal_graph_destroy(self._g))
            self._g = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class VebTree:
    """Standalone device vEB tree (reference veb_tree, veb.cuh:528-1228)."""

    def __init__(self, universe: int, seed: int):
        h = c_void_p()
        _check(load().gal_veb_create(universe, seed, ctypes.byref(h)))
        self._h = h.value
        self.universe = universe
        self.seed = seed

    def close(self) -> None:
        if self._h:
            _check(load().gal_veb_destroy(self._h))
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def num_layers(self) -> int:
        return load().gal_veb_num_layers(self._h)

    def layers(self) -> list[np.ndarray]:
        out = []
        for layer in range(self.num_layers):
            words = load().gal_veb_layer_words(self._h, layer)
            arr = np.empty(words, dtype=np.uint64)
            _check(load().gal_veb_dump(self._h, layer, arr.ctypes.data))
            out.append(arr)
        return out

    def run_ops(self, d_ops: int, n: int, d_results: int, stream: int = 0) -> None:
        _check(load().gal_veb_run_ops(self._h, d_ops, n, d_results, stream))

    def load(self, leaf_words: np.ndarray) -> None:
        """Set the leaf layer (bit i of word w = id 64w + i) and rebuild every
        upper layer as the OR of its children (gal_veb_load)."""
        w = np.ascontiguousarray(leaf_words, dtype=np.uint64)
        _check(load().gal_veb_load(self._h, w.ctypes.data, len(w)))

    def find_batch(self, d_queries: int, n: int, d_out: int, staged: bool = True, stream: int = 0) -> None:
        """d_out[i] = smallest set id >= d_queries[i], or ~0 (gal_veb_find_batch);
        staged: upper layers from a per-CTA shared-memory copy."""
        _check(load().gal_veb_find_batch(self._h, d_queries, n, d_out, 1 if staged else 0, stream))


# -- global allocator (reference global_allocator.cuh:41-97) -----------------
_GLOBAL: Gallatin | None = None


def init_global_allocator(num_bytes: int, seed: int, print_info: bool = True, running_calloc: bool = False) -> Gallatin:
    """Create the process-wide Gallatin<16 MiB, 16, 4096> allocator."""
    global _GLOBAL
    if _GLOBAL is not None:
        _GLOBAL.free_on_device()
    _GLOBAL = Gallatin.generate_on_device(num_bytes, seed, print_info, running_calloc)
    return _GLOBAL


def global_allocator() -> Gallatin:
    if _GLOBAL is None:
        raise GalError("init_global_allocator has not been called")
    return _GLOBAL


def free_global_allocator() -> None:
    global _GLOBAL
    if _GLOBAL is not None:
        _GLOBAL.free_on_device()
        _GLOBAL = None


def print_global_stats() -> None:
    global_allocator().print_info()


# -- host-memory and combined global allocators (global_allocator.cuh:98-183) --
_GLOBAL_HOST: Gallatin | None = None


def init_global_allocator_host(num_bytes: int, seed: int, print_info: bool = True,
                               running_calloc: bool = False) -> Gallatin:
    """Create the process-wide Gallatin<16 MiB, 16, 4096> over pinned host memory."""
    global _GLOBAL_HOST
    if _GLOBAL_HOST is not None:
        _GLOBAL_HOST.free_on_device()
    _GLOBAL_HOST = Gallatin.generate_on_device_host(num_bytes, seed, print_info, running_calloc)
    return _GLOBAL_HOST


def global_host_allocator() -> Gallatin:
    if _GLOBAL_HOST is None:
        raise GalError("init_global_allocator_host has not been called")
    return _GLOBAL_HOST


def free_global_allocator_host() -> None:
    global _GLOBAL_HOST
    if _GLOBAL_HOST is not None:
        _GLOBAL_HOST.free_on_device()
        _GLOBAL_HOST = None


def print_global_stats_host() -> None:
    global_host_allocator().print_info()


def init_global_allocator_combined(num_bytes: int, host_bytes: int, seed: int, print_info: bool = True,
                                   running_calloc: bool = False) -> tuple[Gallatin, Gallatin]:
    """Both the device and the host-memory global allocators."""
    return (init_global_allocator(num_bytes, seed, print_info, running_calloc),
            init_global_allocator_host(host_bytes, seed, print_info, running_calloc))


def free_global_allocator_combined() -> None:
    free_global_allocator()
    free_global_allocator_host()

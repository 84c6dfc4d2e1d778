"""ORACLE — test infrastructure only.

Bindings to the CPU restatement of the reference vEB tree (veb_oracle.c), the
glibc CPU-baseline replay (cpu_replay.c) and, when it has been built, the
reference's own CUDA build (oracle/_ref/libgalref_*.so, from the oracle/ref_*.cu harness).
Only tests/, the smoke check and bench.py's baseline legs use this package;
the product (gallatin_gb300/) never imports it.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_double, c_int, c_int64, c_uint32, c_uint64, c_void_p

import numpy as np

from . import build

VEB_OP_DTYPE = np.dtype([("code", "<u4"), ("tid", "<u4"), ("arg", "<u8"), ("arg2", "<u8")])
FAIL = (1 << 64) - 1
MODE_REFERENCE = 0
MODE_GB300 = 1

_ORACLE = None
_REPLAY = None
_REF = None


def load_oracle():
    global _ORACLE
    if _ORACLE is None:
        build.build_oracle()
        lib = ctypes.CDLL(str(build.oracle_lib()))
        lib.oracle_veb_shape.restype = c_int
        lib.oracle_veb_shape.argtypes = [c_uint64, c_void_p]
        lib.oracle_veb_run.restype = c_int64
        lib.oracle_veb_run.argtypes = [c_uint64, c_uint64, c_int, c_void_p, c_uint64, c_void_p, c_void_p, c_void_p]
        lib.oracle_murmur64a_u64.restype = c_uint64
        lib.oracle_murmur64a_u64.argtypes = [c_uint64, c_uint64]
        _ORACLE = lib
    return _ORACLE


def veb_shape(universe: int) -> list[int]:
    words = np.zeros(8, dtype=np.uint64)
    layers = load_oracle().oracle_veb_shape(universe, words.ctypes.data)
    if layers < 0:
        raise ValueError(f"bad universe {universe}")
    return [int(w) for w in words[:layers]]


def veb_run(universe: int, seed: int, mode: int, ops: np.ndarray):
    """Run ops on a full tree. Returns (results, layers top-first, quirks-so-far per op)."""
    ops = np.ascontiguousarray(ops, dtype=VEB_OP_DTYPE)
    n = len(ops)
    results = np.zeros(n, dtype=np.uint64)
    quirks = np.zeros(n, dtype=np.uint64)
    shape = veb_shape(universe)
    flat = np.zeros(sum(shape), dtype=np.uint64)
    rc = load_oracle().oracle_veb_run(
        universe, seed, mode, ops.ctypes.data, n, results.ctypes.data, flat.ctypes.data, quirks.ctypes.data
    )
    if rc < 0:
        raise ValueError("oracle rejected the arguments")
    layers, off = [], 0
    for w in shape:
        layers.append(flat[off : off + w].copy())
        off += w
    return results, layers, quirks


def murmur64a(key: int, seed: int) -> int:
    return int(load_oracle().oracle_murmur64a_u64(key, seed))


# -- glibc CPU baseline --------------------------------------------------------
def load_replay():
    global _REPLAY
    if _REPLAY is None:
        build.build_oracle()
        lib = ctypes.CDLL(str(build.replay_lib()))
        lib.cpu_replay_mixed.restype = c_double
        lib.cpu_replay_mixed.argtypes = [
            c_uint64, c_uint64, c_uint64, c_uint32, c_uint64, c_void_p, c_uint32, c_uint32, c_uint64, c_uint64,
            c_int, POINTER(c_uint64), POINTER(c_uint64),
        ]
        lib.cpu_replay_pairs.restype = c_double
        lib.cpu_replay_pairs.argtypes = [c_uint64, c_uint64, c_int, POINTER(c_uint64), POINTER(c_uint64)]
        lib.cpu_replay_mixed_zeroed.restype = c_double
        lib.cpu_replay_mixed_zeroed.argtypes = [c_uint64, c_uint64, c_uint64, c_uint32, c_uint64, c_void_p, c_int,
                                                POINTER(c_uint64), POINTER(c_uint64)]
        lib.cpu_replay_fill_drain.restype = c_double
        lib.cpu_replay_fill_drain.argtypes = [c_uint64, c_void_p, c_void_p, c_int, POINTER(c_uint64),
                                              POINTER(c_uint64)]
        lib.cpu_replay_batches.restype = c_double
        lib.cpu_replay_batches.argtypes = [c_void_p, c_void_p, c_uint32, c_void_p, c_int, POINTER(c_uint64)]
        lib.cpu_mixed_classes.restype = None
        lib.cpu_mixed_classes.argtypes = [c_uint64, c_uint32, c_uint64, c_void_p]
        lib.cpu_table.restype = c_double
        lib.cpu_table.argtypes = [c_uint64, c_uint64, c_uint64, c_uint64, c_int, POINTER(c_uint64)]
        lib.cpu_vectors.restype = c_double
        lib.cpu_vectors.argtypes = [c_void_p, c_uint64, c_uint32, c_int, POINTER(c_uint64), POINTER(c_uint64)]
        lib.cpu_serving_checksums.restype = None
        lib.cpu_serving_checksums.argtypes = [c_uint64, c_void_p, c_uint64, c_void_p, c_int]
        lib.cpu_replay_serving.restype = c_double
        lib.cpu_replay_serving.argtypes = [c_uint64, c_void_p, c_void_p, c_void_p, c_uint32, c_uint32, c_uint64,
                                           c_uint64, c_int, c_void_p, c_void_p, POINTER(c_uint64)]
        _REPLAY = lib
    return _REPLAY


def cpu_mixed_classes(n: int, rounds: int, seed: int) -> np.ndarray:
    out = np.empty(n * rounds, dtype=np.uint8)
    load_replay().cpu_mixed_classes(n, rounds, seed, out.ctypes.data)
    return out.reshape(rounds, n)


def cpu_replay_mixed(n, tid_begin, tid_end, rounds, seed, *, seg_every=0, block_dim=256, seg_lo=16 << 20,
                     seg_hi=256 << 20, workers=1, classes: np.ndarray | None = None):
    misses, bad = c_uint64(0), c_uint64(0)
    ptr = classes.ctypes.data if classes is not None else None
    secs = load_replay().cpu_replay_mixed(n, tid_begin, tid_end, rounds, seed, ptr, seg_every, block_dim, seg_lo,
                                          seg_hi, workers, ctypes.byref(misses), ctypes.byref(bad))
    return secs, misses.value, bad.value


def cpu_replay_batches(reqs: np.ndarray, offsets: np.ndarray, table_slots: int, workers: int = 1):
    """glibc malloc/free over the batched request stream; returns (seconds, misses)."""
    reqs = np.ascontiguousarray(reqs, dtype=np.uint64)
    offsets = np.ascontiguousarray(offsets, dtype=np.uint64)
    table = np.zeros(table_slots + 1, dtype=np.uint64)
    misses = c_uint64(0)
    secs = load_replay().cpu_replay_batches(reqs.ctypes.data, offsets.ctypes.data, len(offsets) - 1,
                                            table.ctypes.data, workers, ctypes.byref(misses))
    return secs, misses.value


def cpu_table(n: int, nbuckets: int, table_seed: int = 9, key_seed: int = 42, workers: int = 1):
    """glibc chained table: insert, erase half, compact, reinsert (timed);
    returns (seconds, failures)."""
    bad = c_uint64(0)
    secs = load_replay().cpu_table(n, nbuckets, table_seed, key_seed, workers, ctypes.byref(bad))
    return secs, bad.value


def cpu_vectors(lengths: np.ndarray, start: int = 1, workers: int = 1):
    """glibc doubling vectors; returns (seconds, failures, pushes)."""
    lengths = np.ascontiguousarray(lengths, dtype=np.uint32)
    bad, pushes = c_uint64(0), c_uint64(0)
    secs = load_replay().cpu_vectors(lengths.ctypes.data, len(lengths), start, workers, ctypes.byref(bad),
                                     ctypes.byref(pushes))
    return secs, bad.value, pushes.value


def serving_checksums(tokens: np.ndarray, seed: int, workers: int = 1) -> np.ndarray:
    """The checksum each stream of a serving trace must report when it
    finishes (sum of token * (2 * position + 1) mod 2^64)."""
    tokens = np.ascontiguousarray(tokens, dtype=np.uint32)
    out = np.zeros(len(tokens), dtype=np.uint64)
    load_replay().cpu_serving_checksums(len(tokens), tokens.ctypes.data, seed, out.ctypes.data, workers)
    return out


def cpu_replay_serving(trace: dict, admit_step: np.ndarray, *, page_bytes: int = 8192, seed: int = 42,
                       workers: int = 1):
    """glibc malloc/free through the serving schedule; returns (seconds,
    checksums, latency histogram, NULL count)."""
    tokens = np.ascontiguousarray(trace["tokens"], dtype=np.uint32)
    pages = np.ascontiguousarray(trace["pages"], dtype=np.uint32)
    admit = np.ascontiguousarray(admit_step, dtype=np.uint32)
    n = len(tokens)
    checksum = np.zeros(max(n, 1), dtype=np.uint64)
    hist = np.zeros(864, dtype=np.uint64)
    nulls = c_uint64(0)
    secs = load_replay().cpu_replay_serving(n, tokens.ctypes.data, pages.ctypes.data, admit.ctypes.data,
                                            int(trace["steps"]), int(trace["tokens_per_page"]), page_bytes, seed,
                                            workers, checksum.ctypes.data, hist.ctypes.data, ctypes.byref(nulls))
    return secs, checksum[:n], hist, nulls.value


def cpu_replay_mixed_zeroed(n, tid_begin, tid_end, rounds, seed, *, workers=1, classes: np.ndarray | None = None):
    """The mixed workload through glibc calloc, checking each allocation reads
    zero; returns (seconds, misses, non-zero allocations)."""
    misses, bad = c_uint64(0), c_uint64(0)
    ptr = classes.ctypes.data if classes is not None else None
    secs = load_replay().cpu_replay_mixed_zeroed(n, tid_begin, tid_end, rounds, seed, ptr, workers,
                                                 ctypes.byref(misses), ctypes.byref(bad))
    return secs, misses.value, bad.value


def cpu_replay_fill_drain(classes: np.ndarray, workers: int = 1):
    """glibc malloc for every class of the trace (fill), then verify and free
    (drain); returns (seconds, misses, verify failures)."""
    classes = np.ascontiguousarray(classes, dtype=np.uint8)
    table = np.zeros(len(classes), dtype=np.uint64)
    misses, bad = c_uint64(0), c_uint64(0)
    secs = load_replay().cpu_replay_fill_drain(len(classes), classes.ctypes.data, table.ctypes.data, workers,
                                               ctypes.byref(misses), ctypes.byref(bad))
    return secs, misses.value, bad.value


def cpu_replay_pairs(n, size, workers=1):
    misses, bad = c_uint64(0), c_uint64(0)
    secs = load_replay().cpu_replay_pairs(n, size, workers, ctypes.byref(misses), ctypes.byref(bad))
    return secs, misses.value, bad.value


# -- the reference's own CUDA build -------------------------------------------
def load_ref(build_if_missing: bool = True):
    """The reference harness's entry points (oracle/_ref/libgalref_*.so) as
    attributes of one object, or None when unavailable."""
    global _REF
    if _REF is not None:
        return _REF
    import os

    if os.environ.get("GALLATIN_SKIP_REF"):
        return None  # runs that do not need the reference skip its long build
    override = os.environ.get("GALLATIN_REF_LIB")  # os.pathsep-separated libraries
    if override:
        _REF = _bind_ref([ctypes.CDLL(p) for p in override.split(os.pathsep) if p])
        return _REF
    if build_if_missing and not all(p.exists() for p in build.ref_libs()):
        try:
            build.build_reference()
        except RuntimeError:
            return None
    if not all(p.exists() for p in build.ref_libs()):
        return None
    _REF = _bind_ref([ctypes.CDLL(str(p)) for p in build.ref_libs()])
    return _REF


class _RefEntryPoints:
    """Entry points gathered from the harness's family libraries."""


def _bind_ref(libs):
    vp, u64, u32, i32 = c_void_p, c_uint64, c_uint32, c_int
    sigs = {
        "galref_veb_create": (i32, [u64, u64, POINTER(vp)]),
        "galref_veb_destroy": (i32, [vp]),
        "galref_veb_num_layers": (i32, [vp]),
        "galref_veb_layer_words": (u64, [vp, i32]),
        "galref_veb_dump": (i32, [vp, i32, vp]),
        "galref_veb_run_ops": (i32, [vp, vp, u64, vp, vp]),
        "galref_create": (i32, [u64, u64, u64, u64, u64, POINTER(vp)]),
        "galref_create_host": (i32, [u64, u64, u64, u64, u64, POINTER(vp)]),
        "galref_run_fused": (i32, [vp, vp, u64, u64, vp, vp, u32, vp, vp]),
        "galref_destroy": (i32, [vp]),
        "galref_run_pairs": (i32, [vp, u64, u64, u32, vp, vp]),
        "galref_run_mixed": (i32, [vp, u64, u32, u64, u32, u64, u64, vp, u32, vp, vp]),
        "galref_run_mixed_host": (i32, [vp, u64, u32, u64, u32, u64, u64, vp, u32, vp, vp]),
        "galref_run_batches": (i32, [vp, vp, vp, vp, u32, vp, u32, vp, vp]),
        "galref_run_serving": (i32, [vp, vp, vp, vp, vp]),
        "galref_run_serving_fused": (i32, [vp, vp, vp, vp, vp, vp]),
        "galref_table_op": (i32, [vp, vp, u64, u64, u32, vp, u64, u64, vp, vp]),
        "galref_run_vectors": (i32, [vp, vp, u64, u32, vp, vp]),
    }
    out = _RefEntryPoints()
    for name, (res, args) in sigs.items():
        fn = None
        for lib in libs:
            try:
                fn = getattr(lib, name)
                break
            except AttributeError:
                continue
        if fn is None:
            raise RuntimeError(f"reference harness entry point {name} not found")
        fn.restype = res
        fn.argtypes = args
        setattr(out, name, fn)
    return out


class RefVeb:
    """The reference veb_tree on the GPU (generate_on_device: full tree)."""

    def __init__(self, universe: int, seed: int):
        lib = load_ref()
        if lib is None:
            raise RuntimeError("reference build unavailable")
        h = c_void_p()
        if lib.galref_veb_create(universe, seed, ctypes.byref(h)) != 0:
            raise RuntimeError("galref_veb_create failed")
        self._lib, self._h = lib, h.value

    def run_ops(self, d_ops: int, n: int, d_results: int, stream: int = 0) -> None:
        if self._lib.galref_veb_run_ops(self._h, d_ops, n, d_results, stream) != 0:
            raise RuntimeError("galref_veb_run_ops failed")

    def layers(self) -> list[np.ndarray]:
        out = []
        for layer in range(self._lib.galref_veb_num_layers(self._h)):
            arr = np.empty(self._lib.galref_veb_layer_words(self._h, layer), dtype=np.uint64)
            if self._lib.galref_veb_dump(self._h, layer, arr.ctypes.data) != 0:
                raise RuntimeError("galref_veb_dump failed")
            out.append(arr)
        return out

    def close(self) -> None:
        if self._h:
            self._lib.galref_veb_destroy(self._h)
            self._h = None


class RefGallatin:
    """The reference Gallatin<seg,min,max> on the GPU behind the shared workloads."""

    def __init__(self, max_bytes: int, seed: int, segment_size=16 << 20, min_size=16, max_size=4096, *,
                 host_arena: bool = False):
        """host_arena: the reference's generate_on_device_host (pinned host arena)."""
        lib = load_ref()
        if lib is None:
            raise RuntimeError("reference build unavailable")
        h = c_void_p()
        create = lib.galref_create_host if host_arena else lib.galref_create
        rc = create(max_bytes, seed, segment_size, min_size, max_size, ctypes.byref(h))
        if rc != 0:
            raise RuntimeError(f"galref_create{'_host' if host_arena else ''} failed ({rc})")
        self._lib, self._h = lib, h.value

    def run_fused(self, host, n, seed, d_table, d_stats, *, d_classes=0, phases=3, stream=0):
        """Fill/drain through the reference's fused pattern (device first, then `host`)."""
        rc = self._lib.galref_run_fused(self._h, host._h if host is not None else None, n, seed, d_classes, d_table,
                                        phases, d_stats, stream)
        if rc != 0:
            raise RuntimeError(f"galref_run_fused failed ({rc})")

    def run_pairs(self, n, size, d_stats, block_dim=1024, stream=0):
        if self._lib.galref_run_pairs(self._h, n, size, block_dim, d_stats, stream) != 0:
            raise RuntimeError("galref_run_pairs failed")

    def run_mixed(self, n, rounds, seed, d_stats, *, seg_every=0, seg_lo=16 << 20, seg_hi=256 << 20, d_classes=0,
                  block_dim=256, stream=0):
        if self._lib.galref_run_mixed(self._h, n, rounds, seed, seg_every, seg_lo, seg_hi, d_classes, block_dim,
                                      d_stats, stream) != 0:
            raise RuntimeError("galref_run_mixed failed")

    def run_mixed_host(self, n, rounds, seed, h_classes_ptr, *, seg_every=0, seg_lo=16 << 20, seg_hi=256 << 20,
                       block_dim=256, stream=0):
        out = np.zeros(8, dtype=np.uint64)
        if self._lib.galref_run_mixed_host(self._h, n, rounds, seed, seg_every, seg_lo, seg_hi, h_classes_ptr,
                                           block_dim, out.ctypes.data, stream) != 0:
            raise RuntimeError("galref_run_mixed_host failed")
        return out

    def run_batches(self, d_reqs, d_offsets, offsets, d_table, d_stats, *, persistent=False, stream=0):
        offsets = np.ascontiguousarray(offsets, dtype=np.uint64)
        if self._lib.galref_run_batches(self._h, d_reqs, d_offsets, offsets.ctypes.data, len(offsets) - 1, d_table,
                                        1 if persistent else 0, d_stats, stream) != 0:
            raise RuntimeError("galref_run_batches failed")

    def run_serving(self, trace_ptr, params_ptr, out_ptr, stream=0):
        """The serving loop's plain path (one launch per phase per step) over
        the reference allocator; the params' mode is ignored."""
        return self._lib.galref_run_serving(self._h, trace_ptr, params_ptr, out_ptr, stream)

    def run_serving_fused(self, host, trace_ptr, params_ptr, out_ptr, stream=0):
        """The plain-path serving loop over this allocator first and `host`
        (a host-arena RefGallatin) when it returns NULL; default geometry only."""
        return self._lib.galref_run_serving_fused(self._h, host._h, trace_ptr, params_ptr, out_ptr, stream)

    def table_op(self, heads_ptr, nbuckets, seed, op, n, d_stats, *, d_keys=None, key_seed=42, stream=0):
        """The chained table of gallatin_gb300/structures.cuh over the reference allocator."""
        if self._lib.galref_table_op(self._h, heads_ptr, nbuckets, seed, op, d_keys, n, key_seed, d_stats,
                                     stream) != 0:
            raise RuntimeError("galref_table_op failed")

    def run_vectors(self, d_lengths, n, d_stats, *, start=1, stream=0):
        if self._lib.galref_run_vectors(self._h, d_lengths, n, start, d_stats, stream) != 0:
            raise RuntimeError("galref_run_vectors failed")

    def close(self):
        if self._h:
            self._lib.galref_destroy(self._h)
            self._h = None

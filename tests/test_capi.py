"""The C-ABI library loads and exports every entry point gallatin_gb300.h declares (no GPU needed)."""
from __future__ import annotations

import ctypes
import re

import pytest

from conftest import REPO


def declared_functions() -> list[str]:
    text = (REPO / "include" / "gallatin_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(gal_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for expected in ("gal_create", "gal_destroy", "gal_malloc_batch", "gal_free_batch", "gal_veb_run_ops"):
        assert expected in names
    assert len(names) >= 24


def test_library_exports_every_declared_symbol():
    from gallatin_gb300 import _build

    lib_file = _build.build()
    lib = ctypes.CDLL(str(lib_file))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_package_binds_without_gpu():
    import gallatin_gb300 as gal

    lib = gal.load()
    assert lib.gal_last_error() is not None


def test_invalid_geometry_is_rejected_without_touching_the_gpu():
    import gallatin_gb300 as gal

    # validation happens before any CUDA call
    with pytest.raises(gal.GalError, match="power"):
        gal.Gallatin.generate_on_device(1 << 30, 1, print_info=False, segment_size=3 << 20)
    with pytest.raises(gal.GalError, match="max_size"):
        gal.Gallatin.generate_on_device(1 << 30, 1, print_info=False, min_size=64, max_size=1024)
    with pytest.raises(gal.GalError, match="segment"):
        gal.Gallatin.generate_on_device(1 << 30, 1, print_info=False, segment_size=1 << 20, max_size=4096)


def test_create_ex_rejects_unknown_flags_without_touching_the_gpu():
    import ctypes

    import gallatin_gb300 as gal

    lib = gal.load()
    h = ctypes.c_void_p()
    rc = lib.gal_create_ex(1 << 30, 1, 16 << 20, 16, 4096, 0, 0x80, ctypes.byref(h))
    assert rc == 1 and not h.value
    assert b"flags" in lib.gal_last_error()


def test_veb_batch_entry_points_reject_bad_arguments_without_touching_the_gpu():
    import gallatin_gb300 as gal

    lib = gal.load()
    assert lib.gal_veb_load(None, None, 0) == 1
    assert b"NULL" in lib.gal_last_error()
    assert lib.gal_veb_find_batch(None, None, 1, None, 1, None) == 1
    assert b"NULL" in lib.gal_last_error()
    # the form is checked before the handle is read
    handle = ctypes.create_string_buffer(8)
    assert lib.gal_veb_find_batch(ctypes.addressof(handle), None, 0, None, 2, None) == 1
    assert b"staged" in lib.gal_last_error()


def test_batch_entry_points_check_offsets_width_and_mode_without_touching_the_gpu():
    import numpy as np

    import gallatin_gb300 as gal

    lib = gal.load()
    # a handle that is never read: these checks come before any use of it
    fake = ctypes.create_string_buffer(64)
    h = ctypes.addressof(fake)
    reqs = np.zeros(5, dtype=np.uint64)
    stats = np.zeros(8, dtype=np.uint64)
    bad = np.array([0, 5, 3], dtype=np.uint64)  # batch 1 would be [5, 3)
    good = np.array([0, 3, 5], dtype=np.uint64)

    def host(offsets, width=32, mode=0):
        return lib.gal_run_batches_host(h, reqs.ctypes.data, offsets.ctypes.data, 2, 16, width, mode, 0,
                                        stats.ctypes.data, None)

    assert host(bad) == 1 and b"decrease" in lib.gal_last_error()
    assert host(good, width=12) == 1 and b"width" in lib.gal_last_error()
    assert host(good, mode=3) == 1 and b"mode" in lib.gal_last_error()
    d = reqs.ctypes.data  # device pointers are passed through, never read by the checks
    assert lib.gal_run_batches(h, d, d, bad.ctypes.data, 2, d, 32, 1, 0, d, None) == 1
    assert b"decrease" in lib.gal_last_error()
    graph = ctypes.c_void_p(1)
    assert lib.gal_capture_batches(h, d, d, bad.ctypes.data, 2, d, 32, 0, 0, d, ctypes.byref(graph)) == 1
    assert b"decrease" in lib.gal_last_error() and not graph.value


def test_owns_allocation_is_the_arena_range():
    import gallatin_gb300 as gal

    a = object.__new__(gal.Gallatin)  # the range test needs no device state
    a.arena_base, a.arena_bytes = 1 << 40, 64 << 20
    assert a.owns_allocation(1 << 40) and a.owns_allocation((1 << 40) + (64 << 20) - 16)
    assert not a.owns_allocation((1 << 40) + (64 << 20)) and not a.owns_allocation((1 << 40) - 16)

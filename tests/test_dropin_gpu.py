"""A user program written against the reference's header API builds and runs
against the GB300 drop-in headers and libgallatin_gb300.so."""
from __future__ import annotations

import subprocess

import pytest

from conftest import REPO

pytestmark = pytest.mark.gpu


def test_user_program_against_dropin_headers(cuda, tmp_path):
    from gallatin_gb300 import _build

    lib = _build.build()
    exe = tmp_path / "dropin_user"
    cmd = [
        _build.nvcc_path(), "-std=c++17", "-O2", *_build.ARCH_FLAGS, "-I", str(REPO / "include"),
        str(REPO / "tests" / "cuda" / "dropin_user.cu"), "-o", str(exe),
        "-L", str(lib.parent), "-lgallatin_gb300", "-Xlinker", "-rpath", "-Xlinker", str(lib.parent),
    ]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    proc = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert proc.returncode == 0, proc.stdout + proc.stderr
    assert "DROPIN OK" in proc.stdout
    assert "Gallatin usage stats" in proc.stdout

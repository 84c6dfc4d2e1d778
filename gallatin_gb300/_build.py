"""Build libgallatin_gb300.so in-tree with nvcc for sm_103a.

The three translation units compile in parallel into gallatin_gb300/_build/,
then link into one shared library. No torch types or torch extension
machinery are involved: the library is plain CUDA C++ behind a C ABI.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
REPO_DIR = PKG_DIR.parent
CSRC = PKG_DIR / "csrc"
BUILD_DIR = PKG_DIR / "_build"
LIB_NAME = "libgallatin_gb300.so"
SOURCES = ["capi_host.cu", "capi_run.cu", "capi_veb.cu", "capi_noalloc.cu", "capi_bench.cu", "capi_batch.cu",
           "capi_serve.cu",
           "capi_ds.cu", "capi_spill.cu"]
ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build gallatin_gb300")


def common_flags() -> list[str]:
    return [
        "-std=c++17",
        "-O3",
        "-lineinfo",
        *ARCH_FLAGS,
        "-Xcompiler",
        "-fPIC",
        "-I",
        str(REPO_DIR / "include"),
        "-I",
        str(CSRC),
    ]


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"command failed ({proc.returncode}): {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")


def lib_path() -> Path:
    return BUILD_DIR / LIB_NAME


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _deps() -> list[Path]:
    hdrs = list((REPO_DIR / "include").rglob("*.h")) + list((REPO_DIR / "include").rglob("*.cuh"))
    return hdrs + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + [CSRC / s for s in SOURCES]


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile the library if any source is newer than it; return its path."""
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    out = lib_path()
    if not force and not _stale(out, _deps()):
        return out
    nvcc = nvcc_path()
    flags = common_flags()
    objs = [BUILD_DIR / (Path(s).stem + ".o") for s in SOURCES]
    cmds = [[nvcc, *flags, "-c", str(CSRC / s), "-o", str(o)] for s, o in zip(SOURCES, objs)]
    with ThreadPoolExecutor(max_workers=len(cmds)) as ex:
        list(ex.map(_run, cmds))
    tmp = out.with_suffix(".so.tmp")
    _run([nvcc, *ARCH_FLAGS, "-shared", "-o", str(tmp), *map(str, objs)])
    os.replace(tmp, out)
    if verbose:
        print(f"built {out}")
    return out


def ptxas_report() -> str:
    """Registers / spills of every kernel (nvcc -Xptxas -v), for profiling notes."""
    nvcc = nvcc_path()
    lines = []
    for s in SOURCES:
        proc = subprocess.run(
            [nvcc, *common_flags(), "-Xptxas", "-v", "-c", str(CSRC / s), "-o", os.devnull],
            capture_output=True,
            text=True,
        )
        lines.append(proc.stderr)
    return "\n".join(lines)


if __name__ == "__main__":
    build(force=True, verbose=True)

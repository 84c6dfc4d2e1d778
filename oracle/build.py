"""Build recipe for the oracle and the reference build (test infrastructure).

* oracle/_build/liboracle.so      the C restatement (veb_oracle.c), gcc
* oracle/_build/libcpu_replay.so  the glibc malloc/free trace replay used as
                                  the CPU baseline (cpu_replay.c), gcc
* oracle/_ref/include/...         the reference's hot-path headers, copied
                                  unmodified from the reference checkout (an
                                  install step: the reference is header-only
                                  CUDA, and a machine that runs the GPU
                                  tests need not have the checkout)
* oracle/_ref/libgalref_<family>.so
                                  the harness (ref_core.cu, ref_batches.cu,
                                  ref_serving.cu, ref_ds.cu, ref_fused.cu)
                                  compiled with nvcc against those headers,
                                  one library per family so they build in
                                  parallel

Everything lands in git-ignored folders. A machine of another architecture
rebuilds from the staged headers, since binaries built elsewhere do not run
there. The
reference checkout is read from $GALLATIN_REFERENCE, else /root/reference.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

ORACLE_DIR = Path(__file__).resolve().parent
REPO_DIR = ORACLE_DIR.parent
BUILD_DIR = ORACLE_DIR / "_build"
REF_DIR = ORACLE_DIR / "_ref"
REF_INCLUDE = REF_DIR / "include"
REFERENCE_CHECKOUT = Path(os.environ.get("GALLATIN_REFERENCE", "/root/reference"))
REF_FAMILIES = ["core", "batches", "serving", "ds", "fused"]
# the hot path: the allocator and everything it includes
REF_HEADERS = [
    "alloc_utils.cuh",
    "block.cuh",
    "gallatin.cuh",
    "global_allocator.cuh",
    "memory_table.cuh",
    "murmurhash.cuh",
    "shared_block_storage.cuh",
    "timer.cuh",
    "veb.cuh",
]


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"command failed ({proc.returncode}): {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.exists() and d.stat().st_mtime > t for d in deps)


def oracle_lib() -> Path:
    return BUILD_DIR / "liboracle.so"


def replay_lib() -> Path:
    return BUILD_DIR / "libcpu_replay.so"


def ref_lib(family: str = "core") -> Path:
    return REF_DIR / f"libgalref_{family}.so"


def ref_libs() -> list[Path]:
    return [ref_lib(f) for f in REF_FAMILIES]


def build_oracle(force: bool = False) -> None:
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    cc = os.environ.get("CC", "gcc")
    jobs = []
    src = ORACLE_DIR / "veb_oracle.c"
    if force or _stale(oracle_lib(), [src]):
        jobs.append([cc, "-O2", "-fPIC", "-shared", str(src), "-o", str(oracle_lib())])
    src2 = ORACLE_DIR / "cpu_replay.c"
    if force or _stale(replay_lib(), [src2]):
        jobs.append([cc, "-O3", "-fPIC", "-shared", "-pthread", str(src2), "-o", str(replay_lib())])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(_run, jobs))


def stage_reference() -> bool:
    """Copy the reference's allocator headers, unmodified, into oracle/_ref/include."""
    src_dir = REFERENCE_CHECKOUT / "include" / "gallatin" / "allocators"
    dst_dir = REF_INCLUDE / "gallatin" / "allocators"
    if not src_dir.is_dir():
        return (dst_dir / "gallatin.cuh").exists()
    dst_dir.mkdir(parents=True, exist_ok=True)
    for name in REF_HEADERS:
        src = src_dir / name
        dst = dst_dir / name
        if src.exists() and (not dst.exists() or src.stat().st_mtime > dst.stat().st_mtime):
            shutil.copy2(src, dst)
    return (dst_dir / "gallatin.cuh").exists()


def build_reference(force: bool = False) -> bool:
    """Build oracle/_ref/libgalref_<family>.so if the reference headers are available."""
    if not stage_reference():
        return False
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        return False
    common = [ORACLE_DIR / "ref_common.cuh", *(REPO_DIR / "gallatin_gb300" / "csrc").glob("*.cuh")]
    common += list((REF_INCLUDE / "gallatin" / "allocators").glob("*.cuh"))
    common += list((REPO_DIR / "include").rglob("*.cuh")) + list((REPO_DIR / "include").rglob("*.h"))
    cmds = []
    for family in REF_FAMILIES:
        src = ORACLE_DIR / f"ref_{family}.cu"
        if not force and not _stale(ref_lib(family), [src, *common]):
            continue
        cmds.append([
            nvcc,
            "-std=c++17",
            "-O3",
            "-lineinfo",
            "-gencode",
            "arch=compute_103a,code=sm_103a",
            "-Xcompiler",
            "-fPIC",
            "-shared",
            "-w",
            "-I",
            str(REF_INCLUDE),
            "-I",
            str(REPO_DIR / "include"),
            "-I",
            str(REPO_DIR / "gallatin_gb300" / "csrc"),
            str(src),
            "-o",
            str(ref_lib(family)),
        ])
    with ThreadPoolExecutor(max_workers=max(1, len(cmds))) as ex:
        list(ex.map(_run, cmds))
    return True


if __name__ == "__main__":
    build_oracle(force=True)
    print("reference build:", build_reference(force=True))

"""Build recipe for the CUDA library (sm_103a).

The artefact is built in-tree and git-ignored:
  nexusbvh_gb300/libnxb_gb300.so   kernels + C ABI
Object files go to _build/ at the repository root.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "nexusbvh_gb300"
CSRC = PKG / "csrc"
BUILD = ROOT / "_build"
LIB = PKG / "libnxb_gb300.so"

CUDA_SOURCES = ["setup.cu", "radix_sort.cu", "hploc.cu", "wide.cu", "eval.cu", "capi.cu", "batch.cu", "server.cu", "validate.cu"]
# --use_fast_math matches the reference's compile flags; the numerics the
# tree depends on are pinned in the sources and checked by the self-test.
NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-O3", "--use_fast_math", "-lineinfo", "-std=c++17",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA library cannot be built")


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"command failed ({proc.returncode}): {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_cuda(force: bool = False, verbose_ptxas: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    headers = sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + [ROOT / "include" / "nxb_gb300.h"]
    objs = []
    jobs = []
    for src in CUDA_SOURCES:
        s = CSRC / src
        o = BUILD / (src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            flags = NVCC_FLAGS + (["-Xptxas", "-v"] if verbose_ptxas else [])
            jobs.append([nvcc(), *flags, "-c", str(s), "-o", str(o)])
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(_run, jobs))
    if force or jobs or _stale(LIB, objs):
        tmp = LIB.with_suffix(".so.tmp")
        _run([nvcc(), "-shared", "-cudart", "shared", "-o", str(tmp), *map(str, objs),
              "-Xlinker", "-rpath,/usr/local/cuda/lib64"])
        os.replace(tmp, LIB)
    return LIB


def build_all(force: bool = False) -> None:
    build_cuda(force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print(LIB)

"""Build recipe for the reference's own CUDA build (test infrastructure).

The reference (StokastX/NexusBVH) is a few C++/CUDA translation units with
no build-time code generation; its only external dependency is CUB, which
ships inside the CUDA toolkit (CCCL 3.0.1 with CUDA 13.0).  Its CMake build
is not used: this script compiles the sources directly.

  stage():  copies the reference's source files verbatim from the read-only
            checkout ($NXB_REFERENCE, else a `reference` directory beside
            this repository's checkout) into
            oracle/_ref/src/, plus one patched copy of BinaryBuilder.cu whose
            SEARCH_RADIUS can be set with -D (the reference hard-codes 8).
            oracle/_ref/ is git-ignored: nothing of the reference is
            committed.  The staged copy travels with the working tree to the
            GPU machine, which has no checkout of the reference.
  build():  compiles the staged sources with the reference's flags
            (--use_fast_math -rdc=true; arch sm_103, which is what `native` resolves to
            on GB300) plus oracle/ref_harness.cpp into
            oracle/_ref/libnxbref_r{4,8,16}.so, one per search radius.
  build_auction():  copies the reference's auction slot assignment
            (AuctionAssignment, the USE_AUCTION cost table of the BVH8
            kernel, the nibble helpers) verbatim into oracle/_ref/*.inc and
            compiles them as host code with oracle/ref_auction.cpp into
            oracle/_ref/libref_auction.so (g++ only; no GPU involved).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

ORACLE_DIR = Path(__file__).resolve().parent
REF_OUT = ORACLE_DIR / "_ref"
STAGE = REF_OUT / "src"
OBJ = REF_OUT / "obj"
RADII = (8, 16, 4)
FILES = [
    "NexusBVH/include/NXB/AABB.h", "NexusBVH/include/NXB/BVH.h", "NexusBVH/include/NXB/BVHBuilder.h",
    "NexusBVH/include/NXB/BVHBuildMetrics.h", "NexusBVH/include/NXB/BuildConfig.h",
    "NexusBVH/include/NXB/Triangle.h", "NexusBVH/include/NXB/Math/CudaMath.h",
    "NexusBVH/src/BVHBuilder.cpp", "NexusBVH/src/Math/Math.h",
    "NexusBVH/src/Cuda/BinaryBuilder.cu", "NexusBVH/src/Cuda/BinaryBuilder.h",
    "NexusBVH/src/Cuda/BuildState.h", "NexusBVH/src/Cuda/BuilderUtils.h", "NexusBVH/src/Cuda/CudaUtils.h",
    "NexusBVH/src/Cuda/Eval.cu", "NexusBVH/src/Cuda/Eval.h", "NexusBVH/src/Cuda/Setup.cu",
    "NexusBVH/src/Cuda/Setup.h", "NexusBVH/src/Cuda/WideConverter.cu", "NexusBVH/src/Cuda/WideConverter.h",
]
ARCH = ["-gencode", "arch=compute_103,code=sm_103"]


def reference_root() -> Path:
    env = os.environ.get("NXB_REFERENCE")
    if env:
        return Path(env)
    return ORACLE_DIR.parent.parent / "reference"  # a checkout beside this repository's


def lib_path(radius: int = 8) -> Path:
    return REF_OUT / f"libnxbref_r{radius}.so"


def stage() -> bool:
    src = reference_root()
    if not (src / "NexusBVH").is_dir():
        return (STAGE / "NexusBVH").is_dir()
    for f in FILES:
        dst = STAGE / f
        dst.parent.mkdir(parents=True, exist_ok=True)
        if not dst.exists() or dst.read_bytes() != (src / f).read_bytes():
            shutil.copyfile(src / f, dst)
    bb = (src / "NexusBVH/src/Cuda/BinaryBuilder.cu").read_text()
    patched = bb.replace("#define SEARCH_RADIUS 8", "#ifndef SEARCH_RADIUS\n#define SEARCH_RADIUS 8\n#endif", 1)
    if patched == bb:
        raise RuntimeError("SEARCH_RADIUS definition not found in BinaryBuilder.cu")
    p = STAGE / "NexusBVH/src/Cuda/BinaryBuilder_radius.cu"
    if not p.exists() or p.read_text() != patched:
        p.write_text(patched)
    return True


def _run(cmd):
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"reference build step failed: {' '.join(map(str, cmd))}\n{proc.stderr[-4000:]}")


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and Path(c).exists():
            return c
    raise RuntimeError("nvcc not found")


def build(force: bool = False) -> list[Path]:
    if not stage():
        return []
    nvcc = _nvcc()
    OBJ.mkdir(parents=True, exist_ok=True)
    inc = ["-I", str(STAGE / "NexusBVH/include"), "-I", str(STAGE / "NexusBVH/src")]
    cu = [nvcc, *ARCH, "--use_fast_math", "-rdc=true", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", *inc]
    units = {
        "BVHBuilder.o": ["g++", "-O2", "-std=c++17", "-fPIC", *inc, "-I/usr/local/cuda/include", "-c",
                         str(STAGE / "NexusBVH/src/BVHBuilder.cpp")],
        "Setup.o": cu + ["-c", str(STAGE / "NexusBVH/src/Cuda/Setup.cu")],
        "WideConverter.o": cu + ["-c", str(STAGE / "NexusBVH/src/Cuda/WideConverter.cu")],
        "Eval.o": cu + ["-c", str(STAGE / "NexusBVH/src/Cuda/Eval.cu")],
        "harness.o": ["g++", "-O2", "-std=c++17", "-fPIC", *inc, "-I/usr/local/cuda/include", "-c",
                      str(ORACLE_DIR / "ref_harness.cpp")],
        "BinaryBuilder_r8.o": cu + ["-c", str(STAGE / "NexusBVH/src/Cuda/BinaryBuilder.cu")],
    }
    for r in RADII:
        if r != 8:
            units[f"BinaryBuilder_r{r}.o"] = cu + [f"-DSEARCH_RADIUS={r}", "-c",
                                                   str(STAGE / "NexusBVH/src/Cuda/BinaryBuilder_radius.cu")]
    jobs = []
    for name, cmd in units.items():
        out = OBJ / name
        srcs = [Path(a) for a in cmd if a.endswith((".cu", ".cpp"))]
        if force or not out.exists() or any(s.stat().st_mtime > out.stat().st_mtime for s in srcs):
            jobs.append(cmd + ["-o", str(out)])
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(_run, jobs))
    libs = []
    common = [OBJ / n for n in ("BVHBuilder.o", "Setup.o", "WideConverter.o", "Eval.o", "harness.o")]
    for r in RADII:
        lib = lib_path(r)
        objs = common + [OBJ / f"BinaryBuilder_r{r}.o"]
        if force or jobs or not lib.exists():
            _run([nvcc, *ARCH, "-shared", "-cudart", "shared", "-o", str(lib), *map(str, objs),
                  "-Xlinker", "-rpath,/usr/local/cuda/lib64"])
        libs.append(lib)
    return libs


def _braced(text: str, start: int) -> int:
    """Index just past the brace block that opens at or after `start`."""
    i = text.index("{", start)
    depth = 0
    for k in range(i, len(text)):
        if text[k] == "{":
            depth += 1
        elif text[k] == "}":
            depth -= 1
            if depth == 0:
                return k + 1
    raise RuntimeError("unbalanced braces")


def auction_lib() -> Path:
    return REF_OUT / "libref_auction.so"


def build_auction(force: bool = False) -> Path | None:
    """The reference's auction assignment as a host library (see above);
    None when the reference's sources are not available."""
    if not stage():
        return None
    wide = (STAGE / "NexusBVH/src/Cuda/WideConverter.cu").read_text()
    utils = (STAGE / "NexusBVH/src/Cuda/BuilderUtils.h").read_text()
    # the file's constants (INVALID_ASSIGNMENT, THETA, MAX_COST, invTheta, ...)
    # then GetCost (both overloads), ComputeAssignmentCost, AuctionAssignment
    p0 = wide.index("#define INVALID_ASSIGNMENT")
    p1 = wide.index("namespace NXB", p0)
    a = wide.index("__device__ __forceinline__ float GetCost(uint32_t s, float3 offset)")
    b = _braced(wide, wide.index("void AuctionAssignment("))
    functions = "}  // namespace NXB\n" + wide[p0:p1] + "namespace NXB {\n" + wide[a:b]
    # the kernel's cost table and call, from its parent centroid to the call
    c = wide.index("float3 parentCentroid =")
    d = wide.index("#else", wide.index("#ifdef USE_AUCTION", c))
    table = "\n".join(line for line in wide[c:d].splitlines() if not line.strip().startswith("#ifdef"))
    e = utils.index("__device__ __forceinline__ uint32_t GetNibble(")
    f = _braced(utils, utils.index("void SetNibble(", e))
    nibbles = utils[e:f]
    REF_OUT.mkdir(parents=True, exist_ok=True)
    outs = {"auction_functions.inc": functions, "auction_cost_table.inc": table, "auction_nibbles.inc": nibbles}
    changed = force or not auction_lib().exists()
    for name, body in outs.items():
        p = REF_OUT / name
        if not p.exists() or p.read_text() != body:
            p.write_text(body)
            changed = True
    src = ORACLE_DIR / "ref_auction.cpp"
    if changed or src.stat().st_mtime > auction_lib().stat().st_mtime:
        cxx = os.environ.get("CXX", "g++")
        _run([cxx, "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
              "-I", str(ORACLE_DIR), "-o", str(auction_lib()), str(src)])
    return auction_lib()


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
    print(build_auction(force="--force" in sys.argv))

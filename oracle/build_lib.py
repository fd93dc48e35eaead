"""Build recipe for the CPU oracle (test infrastructure, never shipped).

  oracle/liboracle.so   the C++ restatement of the pipeline (g++, no
                        contraction, no fast-math)
The reference's own CUDA build (oracle/_ref/) has its own recipe in
oracle/build_ref.py.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

ORACLE_DIR = Path(__file__).resolve().parent
ORACLE_LIB = ORACLE_DIR / "liboracle.so"


def build_oracle(force: bool = False) -> Path:
    src = ORACLE_DIR / "nxb_oracle.cpp"
    if force or not ORACLE_LIB.exists() or src.stat().st_mtime > ORACLE_LIB.stat().st_mtime:
        tmp = ORACLE_LIB.with_suffix(".so.tmp")
        cxx = os.environ.get("CXX", "g++")
        cmd = [cxx, "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", "-ffp-contract=off",
               "-fno-fast-math", "-o", str(tmp), str(src)]
        proc = subprocess.run(cmd, capture_output=True, text=True)
        if proc.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{proc.stderr}")
        os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))

"""Build recipe of the oracle (test infrastructure): oracle/liboracle.so.

Compiled with -ffp-contract=off so float arithmetic is not fused, matching the
reference's C# evaluation (aarch64 gcc fuses by default otherwise).
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "liboracle.so"
SOURCES = [HERE / "bepu_oracle.cpp"]
DEPS = SOURCES + [HERE / "bepu_oracle.h", HERE / "bepu_math.h", HERE / "bepu_oracle_joints.inc",
                  HERE / "bepu_oracle_collide.inc", HERE / "permutation_primes.inc",
                  HERE.parent / "include" / "bepugpu.h"]


def build() -> str:
    if OUT.exists() and all(d.stat().st_mtime <= OUT.stat().st_mtime for d in DEPS):
        return str(OUT)
    cxx = os.environ.get("CXX", "g++")
    cmd = [cxx, "-O3", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread",
           *map(str, SOURCES), "-o", str(OUT)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return str(OUT)


if __name__ == "__main__":
    print(build())

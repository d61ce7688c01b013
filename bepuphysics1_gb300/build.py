"""Builds the native libraries in-tree.

    libbepugpu.so     the GB300 solver behind include/bepugpu.h (sm_103a only)
    libbepuscenes.so  the seeded scene and contact source (include/bepuscenes.h)

Translation units compile in parallel; a library is rebuilt only when one of
its sources is newer than it.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIB_DIR = PKG / "lib"
OBJ_DIR = PKG / "lib" / "obj"

NVCC = os.environ.get("NVCC", "nvcc")
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false: the reference (C#) never fuses a*b+c, and the solver restates
# its arithmetic in the same evaluation order.  Division and sqrt stay IEEE
# (nvcc's defaults -prec-div=true -prec-sqrt=true, -ftz=false).
NVCC_FLAGS = ["-O3", "-lineinfo", "-fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-O2", "-Xcompiler", "-ffp-contract=off"] + GENCODE
CXX = os.environ.get("CXX", "g++")
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall"]

HEADERS = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted((ROOT / "include").glob("*.h"))


def _newer(target: Path, sources) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(s).stat().st_mtime > t for s in sources)


def _run(cmds):
    procs = [(c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)) for c in cmds]
    for c, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError(f"build failed: {' '.join(map(str, c))}\n{out}")


def build(verbose: bool = False) -> dict:
    LIB_DIR.mkdir(parents=True, exist_ok=True)
    OBJ_DIR.mkdir(parents=True, exist_ok=True)
    gpu_lib = LIB_DIR / "libbepugpu.so"
    scene_lib = LIB_DIR / "libbepuscenes.so"
    cu_units = sorted(CSRC.glob("*.cu"))
    cpp_units = [CSRC / "colouring.cpp"]
    compile_cmds, objs = [], []
    for src in cu_units:
        obj = OBJ_DIR / (src.stem + ".o")
        objs.append(obj)
        if _newer(obj, [src, *HEADERS]):
            compile_cmds.append([NVCC, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)])
    for src in cpp_units:
        obj = OBJ_DIR / (src.stem + ".o")
        objs.append(obj)
        if _newer(obj, [src, *HEADERS]):
            compile_cmds.append([CXX, *CXX_FLAGS, "-c", str(src), "-o", str(obj)])
    scene_src = CSRC / "scenes.cpp"
    scene_cmd = None
    if _newer(scene_lib, [scene_src, *HEADERS]):
        scene_cmd = [CXX, *CXX_FLAGS, "-shared", str(scene_src), "-o", str(scene_lib)]
    _run(compile_cmds + ([scene_cmd] if scene_cmd else []))
    if compile_cmds or _newer(gpu_lib, objs):
        _run([[NVCC, *GENCODE, "-shared", *map(str, objs), "-o", str(gpu_lib), "-lcudart"]])
    if verbose:
        print(f"built {gpu_lib} and {scene_lib}")
    return {"gpu": str(gpu_lib), "scenes": str(scene_lib)}


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)

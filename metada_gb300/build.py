"""Build recipes for the CUDA library (sm_103a) and the CPU oracle.

The library is built in-tree: objects in ``metada_gb300/_build/``, the
shared object in ``metada_gb300/_lib/libmetada_gb300.so``.  Translation
units compile in parallel; one ``-gencode`` (sm_103a) only.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD_DIR = PKG / "_build"
LIB_DIR = PKG / "_lib"
LIB_PATH = LIB_DIR / "libmetada_gb300.so"
ORACLE_DIR = ROOT / "oracle"
ORACLE_LIB = ORACLE_DIR / "_build" / "liboracle.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "-Xcompiler",
    "-fPIC",
    "-I",
    str(ROOT / "include"),
    "-I",
    str(CSRC),
]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found (set NVCC or put the CUDA toolkit on PATH)")


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"command failed ({proc.returncode}): {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")


def _stale(target: Path, sources: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(s.stat().st_mtime > t for s in sources)


def build_library(force: bool = False, jobs: int | None = None) -> Path:
    """Compile every ``csrc/*.cu`` for sm_103a and link the shared library."""
    nvcc = _nvcc()
    BUILD_DIR.mkdir(exist_ok=True)
    LIB_DIR.mkdir(exist_ok=True)
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted((ROOT / "include").glob("*.h"))
    units = sorted(CSRC.glob("*.cu"))
    objs = []
    todo = []
    for cu in units:
        obj = BUILD_DIR / (cu.stem + ".o")
        objs.append(obj)
        if force or _stale(obj, [cu] + headers):
            todo.append([nvcc, *NVCC_FLAGS, "-c", str(cu), "-o", str(obj)])
    if todo:
        with ThreadPoolExecutor(max_workers=jobs or min(len(todo), os.cpu_count() or 4)) as ex:
            for fut in [ex.submit(_run, c) for c in todo]:
                fut.result()
    if force or todo or _stale(LIB_PATH, objs):
        _run([nvcc, *ARCH, "-shared", "-o", str(LIB_PATH), *map(str, objs)])
    return LIB_PATH


def build_oracle(force: bool = False) -> Path:
    """Compile the CPU oracle (test infrastructure) with g++ and OpenMP."""
    src = ORACLE_DIR / "oracle.cpp"
    ORACLE_LIB.parent.mkdir(exist_ok=True)
    if force or _stale(ORACLE_LIB, [src, ORACLE_DIR / "oracle.h"]):
        cxx = os.environ.get("CXX", "g++")
        _run([cxx, "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
              str(src), "-o", str(ORACLE_LIB)])
    return ORACLE_LIB


def reference_root() -> Path | None:
    """The reference source tree named by METADA_REFERENCE (None when the
    variable is unset).  A set variable that does not name a tree with a
    ``src/`` directory is an error, not a silent skip."""
    val = os.environ.get("METADA_REFERENCE")
    if not val:
        return None
    ref = Path(val)
    if not (ref / "src").is_dir():
        raise RuntimeError(f"METADA_REFERENCE={val} does not name the reference tree (no src/ there)")
    return ref


def build_reference_harness() -> Path | None:
    """Build the reference-header harness (test infrastructure) from the tree
    that METADA_REFERENCE names; None, with nothing built, when it is unset."""
    ref = reference_root()
    if ref is None:
        return None
    _run(["bash", str(ORACLE_DIR / "build_ref.sh"), str(ref)])
    return ORACLE_DIR / "_ref" / "ref_harness"

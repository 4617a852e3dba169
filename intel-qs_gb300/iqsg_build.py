"""Build libiqsg.so (the CUDA kernels + C ABI) in-tree with nvcc, for sm_103a only.

Each .cu under intel-qs_gb300/csrc compiles to an object in parallel, then nvcc links the
shared library into the iqs_gb300 package directory, where iqs_gb300._lib loads it.
Objects go to intel-qs_gb300/_build (git-ignored).
A rebuild happens only when a source or header is newer than the library.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

ROOT = Path(__file__).resolve().parent     # intel-qs_gb300/
PKG_DIR = ROOT / "iqs_gb300"               # the Python package that loads the library
REPO = ROOT.parent
CSRC = ROOT / "csrc"
INCLUDE = REPO / "include"
BUILD = ROOT / "_build"
LIB = PKG_DIR / "libiqsg.so"
QASM_SRC = ROOT / "qasm" / "iqsg_qasm.cpp"
QASM = PKG_DIR / "iqsg_qasm"                 # QASM front end over the C++ drop-in header

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off", "--expt-relaxed-constexpr",
              "-Xptxas", "-warn-spills"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libiqsg")
    return cand


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))
    return any(p.stat().st_mtime > t for p in deps)


def build_qasm() -> Path:
    """Compile the QASM front end (plain C++ over include/iqs_gb300/qureg.hpp and libiqsg.so)."""
    deps = [QASM_SRC, LIB, *INCLUDE.rglob("*.h"), *INCLUDE.rglob("*.hpp")]
    if QASM.exists() and all(p.stat().st_mtime <= QASM.stat().st_mtime for p in deps):
        return QASM
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        raise RuntimeError("g++ not found: needed for the QASM front end")
    cmd = [cxx, "-std=c++17", "-O2", "-I", str(INCLUDE), str(QASM_SRC), "-L", str(PKG_DIR), "-liqsg",
           "-Wl,-rpath,$ORIGIN", "-o", str(QASM)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"g++ failed on {QASM_SRC.name}:\n{r.stdout}\n{r.stderr}")
    return QASM


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile every CUDA source and link libiqsg.so. Returns the library path."""
    if not force and not _stale():
        return LIB
    BUILD.mkdir(parents=True, exist_ok=True)
    cc = nvcc()

    def compile_one(src: Path) -> Path:
        obj = BUILD / (src.stem + ".o")
        extra = os.environ.get("IQSG_NVCC_EXTRA", "").split()  # e.g. -DIQSG_DFS_MIN_BLOCKS_K3=3
        cmd = [cc, *ARCH, *NVCC_FLAGS, *extra, "-I", str(INCLUDE), "-I", str(CSRC), "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)
        return obj

    srcs = sources()
    with ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
    print(build_qasm())

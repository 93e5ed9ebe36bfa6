"""In-tree build of the CUDA library ``liblbm_gb300.so`` (sm_103a only).

Each translation unit under ``csrc/`` is compiled in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a`` and linked into
``lbmminiapp_gb300/liblbm_gb300.so`` (CUDA runtime linked statically, C ABI of
``include/lbm_gb300.h``).  Rebuilds only when a source or header is newer than
the library.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "liblbm_gb300.so"
APP = PKG / "lbm-gb300-app"

SOURCES = [
    "lbm_api.cu",
    "lbm_step_q19_f64.cu",
    "lbm_step_q19_low.cu",
    "lbm_step_q27_f64.cu",
    "lbm_step_q27_low.cu",
    "lbm_noalloc.cu",
    "lbm_sparse.cu",
    "lbm_compact.cu",
    "lbm_adjoint.cu",
]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr"]


def nvcc() -> str:
    path = shutil.which("nvcc")
    if path:
        return path
    cand = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "bin" / "nvcc"
    if cand.exists():
        return str(cand)
    raise RuntimeError("nvcc not found (set CUDA_HOME)")


def _inputs():
    files = [CSRC / s for s in SOURCES]
    files += sorted(CSRC.glob("*.cuh"))
    files.append(PKG / "app" / "lbm_app.cpp")
    files.append(ROOT / "include" / "lbm_gb300.h")
    return files


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _inputs())


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and up_to_date():
        if not APP.exists():
            build_app()
        return LIB
    BUILD.mkdir(exist_ok=True)
    cc = nvcc()

    def compile_one(src: str) -> Path:
        obj = BUILD / (Path(src).stem + ".o")
        cmd = [cc, *ARCH, *NVCC_FLAGS, "-I", str(ROOT / "include"), "-c", str(CSRC / src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB.with_name(LIB.name + f".tmp{os.getpid()}")
    cmd = [cc, *ARCH, "-shared", "-Xcompiler", "-fPIC", *map(str, objs), "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    build_app()
    return LIB


def build_app() -> Path:
    """The C++ drop-in driver (app/lbm_app.cpp), linked against the library
    with an $ORIGIN rpath so it runs from the package directory."""
    src = PKG / "app" / "lbm_app.cpp"
    tmp = APP.with_name(APP.name + f".tmp{os.getpid()}")
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-I", str(ROOT / "include"), str(src),
           "-L", str(PKG), "-llbm_gb300", "-Wl,-rpath,$ORIGIN", "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"app build failed:\n{r.stderr}")
    os.replace(tmp, APP)
    return APP


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(LIB)

"""Builds the native libraries in-tree.

* ``pipeline_gb300/_lib/libdpcull.so`` -- the CUDA backend (C ABI of include/dpcull.h),
  compiled for sm_103a only, one translation unit per nvcc process, in parallel.
* ``pipeline_gb300/_lib/libdpcull_mgr.so`` -- the C++ ``dp::culling::cuda::Manager`` /
  ``Tree`` host layer over that C ABI.

Floating point: ``--fmad=false -ftz=false -prec-div=true -prec-sqrt=true``.  The exact
culling arithmetic does not depend on these (it uses explicit ``__fmul_rn`` /
``__fadd_rn``), they only make sure no other arithmetic is contracted or flushed.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
CPP = PKG / "cpp"
LIB = PKG / "_lib"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "--fmad=false", "-ftz=false", "-prec-div=true",
              "-prec-sqrt=true", "-std=c++17", "-Xcompiler", "-fPIC", "-I", str(ROOT / "include")]
CU_SOURCES = ["api.cu", "cull.cu", "xform.cu", "bbox.cu", "noalloc.cu", "serve.cu"]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libdpcull")
    return exe


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _stale(out: Path, inputs: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(p.stat().st_mtime > t for p in inputs)


def build_cuda(force: bool = False, verbose: bool = False) -> Path:
    LIB.mkdir(exist_ok=True)
    out = LIB / "libdpcull.so"
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [ROOT / "include" / "dpcull.h"]
    srcs = [CSRC / s for s in CU_SOURCES]
    if not force and not _stale(out, srcs + headers):
        return out
    objdir = LIB / "obj"
    objdir.mkdir(exist_ok=True)
    exe = nvcc()

    def compile_one(src: Path) -> Path:
        obj = objdir / (src.stem + ".o")
        if force or _stale(obj, [src] + headers):
            cmd = [exe, *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
            _run(cmd)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = out.with_suffix(".so.tmp")
    _run([exe, *ARCH, "-shared", "-o", str(tmp), *map(str, objs)])
    os.replace(tmp, out)
    return out


def build_manager(force: bool = False) -> Path | None:
    """C++ Manager/Tree host layer (links against libdpcull.so)."""
    srcs = sorted(CPP.glob("*.cpp"))
    if not srcs:
        return None
    out = LIB / "libdpcull_mgr.so"
    headers = list(CPP.glob("*.h")) + [ROOT / "include" / "dpcull.h"]
    if not force and not _stale(out, srcs + headers + [LIB / "libdpcull.so"]):
        return out
    cxx = shutil.which("g++") or "g++"
    tmp = out.with_suffix(".so.tmp")
    _run([cxx, "-std=c++17", "-O2", "-fPIC", "-shared", "-I", str(ROOT / "include"), "-I", str(CPP),
          *map(str, srcs), "-o", str(tmp), "-L", str(LIB), "-ldpcull", "-Wl,-rpath,$ORIGIN"])
    os.replace(tmp, out)
    return out


def build_all(force: bool = False, verbose: bool = False) -> None:
    build_cuda(force=force, verbose=verbose)
    build_manager(force=force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv, verbose=True)
    print(LIB)

"""Builds libgbh.so (the CUDA library behind include/gbh.h) for sm_103a with nvcc.

Each translation unit gets its own floating-point flags:
  tree.cu  -fmad=false   FP64 keys, moments, FP64 walk, direct sum and kick/drift keep the
                         reference's rounded multiply-then-add order (bit-exact parity);
  walk.cu  fast FP32     FMA contraction on, approximate FP32 division and square root;
  walk_lists.cu          the list walk, with the flags of walk.cu;
  moments.cu             FP32 node moments for the FP32 walks (FMA on, IEEE FP32 division);
  api.cu                 host code;
  noalloc.cu             the entry point whose temporaries live in a static device array;
  split.cu   -fmad=false the hole-aware split step (bit-exact with the CPU restatement);
  adjoint.cu -fmad=false the adjoint pair: FP64 pair kernels bit-exact with the CPU
                         restatement, FP32 pair kernels with explicit fmaf/rsqrtf.
Objects compile in parallel; the shared library links the CUDA runtime statically.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB_PATH = os.path.join(OUT_DIR, "libgbh.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]
UNITS = {
    "tree.cu": ["-fmad=false"],
    "walk.cu": ["-prec-div=false", "-prec-sqrt=false", "-ftz=true"],
    "walk_lists.cu": ["-prec-div=false", "-prec-sqrt=false", "-ftz=true"],
    "moments.cu": [],
    "api.cu": [],
    "noalloc.cu": [],
    "adjoint.cu": ["-fmad=false"],
    "split.cu": ["-fmad=false"],
}


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: libgbh needs the CUDA toolkit to build")
    return path


def _sources_newer(target: str) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps += [os.path.join(HERE, "..", "include", "gbh.h"), __file__]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> str:
    """Compiles libgbh.so in-tree (gravitas_gb300/_lib) and returns its path."""
    if not force and not _sources_newer(LIB_PATH):
        return LIB_PATH
    os.makedirs(OUT_DIR, exist_ok=True)
    cc = nvcc()
    extra = list(extra or [])

    def compile_unit(item):
        src, flags = item
        obj = os.path.join(OUT_DIR, src.replace(".cu", ".o"))
        cmd = [cc, *ARCH, *COMMON, *flags, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr, file=sys.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_unit, UNITS.items()))
    tmp = LIB_PATH + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-ldl"]  # NVTX3 loads a profiler's hooks with dlopen
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    v = "-v" in sys.argv
    extra = ["-Xptxas", "-v"] if "--ptxas" in sys.argv else None
    print(build(force=True, verbose=v or bool(extra), extra=extra))

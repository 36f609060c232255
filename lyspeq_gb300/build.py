"""Build the engine's shared library, lyspeq_gb300/liblqg.so, for sm_103a.

Each CUDA translation unit is compiled by nvcc in parallel, then linked into
one shared library that exports the C ABI of include/lqg.h.  Objects go to
lyspeq_gb300/_build/.  Run: python -m lyspeq_gb300.build
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "liblqg.so")
# Self-checking variant (-DLQG_CHECKED): device index checks that count and skip
# out-of-bounds accesses instead of performing them.
CHECKED_BUILD = os.path.join(HERE, "_build_checked")
CHECKED_LIB = os.path.join(HERE, "liblqg_checked.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["lqg_api.cu", "lqg_fisher.cu", "k_fp64.cu", "k_factor.cu", "k_accum.cu", "k_tc.cu",
           "lqg_noalloc.cu", "lqg_reso.cu", "lqg_tables.cu",
           "lqg_boot.cu", "lqg_smooth.cu", "lqg_probe.cu"]


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(src: str, nvcc: str, extra: list, build_dir: str = BUILD) -> str:
    obj = os.path.join(build_dir, os.path.basename(src) + ".o")
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [
        os.path.join(HERE, "..", "include", "lqg.h")]
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "-Xptxas", "-warn-spills", *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False, extra: list | None = None, checked: bool = False) -> str:
    bdir, lib = (CHECKED_BUILD, CHECKED_LIB) if checked else (BUILD, LIB)
    os.makedirs(bdir, exist_ok=True)
    nvcc = nvcc_path()
    extra = list(extra or []) + (["-DLQG_CHECKED"] if checked else [])
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, nvcc, extra, bdir), SOURCES))
    newest = max(os.path.getmtime(o) for o in objs)
    if not os.path.exists(lib) or os.path.getmtime(lib) < newest:
        cmd = [nvcc, *ARCH, "-shared", "-o", lib, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(lib)
    return lib


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if a != "--checked"]
    build(verbose=True, extra=args, checked="--checked" in sys.argv[1:])

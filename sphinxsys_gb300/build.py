"""In-tree build of libsphx_cuda.so for sm_103a (nvcc, one translation unit per source,
compiled in parallel, linked with -shared).  Output: sphinxsys_gb300/_build/; the
bounds-checked build (-DSPHX_CHECK: index tests in the kernels, read with
sphx_check_violations) goes to sphinxsys_gb300/_build_check/."""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libsphx_cuda.so")
OUT_DIR_CHECK = os.path.join(HERE, "_build_check")
LIB_CHECK = os.path.join(OUT_DIR_CHECK, "libsphx_cuda.so")
SOURCES = ["sphx_core.cu", "cell_list.cu", "relation.cu", "fluid.cu", "mixed.cu", "batch.cu", "ck.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-I", os.path.join(ROOT, "include")]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _headers_mtime() -> float:
    paths = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    paths.append(os.path.join(ROOT, "include", "sphx", "sphx.h"))
    return max(os.path.getmtime(p) for p in paths)


def _compile(src: str, extra: list, out_dir: str = OUT_DIR) -> str:
    obj = os.path.join(out_dir, os.path.splitext(src)[0] + ".o")
    s = os.path.join(CSRC, src)
    if os.path.exists(obj) and os.path.getmtime(obj) > max(os.path.getmtime(s), _headers_mtime()):
        return obj
    cmd = [nvcc()] + ARCH + FLAGS + extra + ["-c", s, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False, extra: list = None, checked: bool = False) -> str:
    out_dir, lib = (OUT_DIR_CHECK, LIB_CHECK) if checked else (OUT_DIR, LIB)
    os.makedirs(out_dir, exist_ok=True)
    extra = list(extra or []) + (["-DSPHX_CHECK"] if checked else [])
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra, out_dir), SOURCES))
    if not os.path.exists(lib) or os.path.getmtime(lib) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", lib] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(lib)
    return lib


if __name__ == "__main__":
    args = sys.argv[1:]
    build(verbose=True, extra=[a for a in args if a != "--checked"], checked="--checked" in args)

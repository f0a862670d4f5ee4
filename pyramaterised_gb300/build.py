"""Build the engine's C-ABI shared library (``lib/libpqc_gb300.so``) with nvcc.

The library is built in-tree for sm_103a only (GB300).  Translation units are
compiled in parallel; objects go to ``_build/``.  Run ``python -m
pyramaterised_gb300.build`` (or ``__graft_entry__.build()``).
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIBNAME = "libpqc_gb300.so"
SOURCES = ["sweep_df_a.cu", "sweep_df_b.cu", "sweep_df_dual.cu", "sweep_f32.cu", "sweep_f64.cu", "multi.cu",
           "adjoint.cu", "measures.cu", "gram_tc.cu", "program.cu", "sweep.cu", "plain.cu", "noalloc.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall"]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def lib_path():
    return os.path.join(LIBDIR, LIBNAME)


def _compile(src):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc()] + ARCH + FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    out = lib_path()
    tmp = out + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, out)
    if verbose:
        print("built", out)
    return out


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)

"""Builds libestl_cuda.so (the C-ABI FFT engine) in-tree with nvcc for sm_103a.

Translation units are compiled in parallel; an object is rebuilt only when a
source or header of the package is newer than it.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libestl_cuda.so")

SOURCES = [
    "kernels_single.cu",
    "kernels_col.cu",
    "kernels_row.cu",
    "planner.cpp",
    "tuner.cu",
    "api.cu",
    "noalloc.cu",
    "conv_plan.cpp",
    "conv.cu",
    "conv2d.cu",
    "packed_plan.cpp",
    "packed.cu",
    "serve.cu",
]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
         "--expt-relaxed-constexpr", "-I", CSRC, "-I", os.path.join(ROOT, "include")]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libestl_cuda.so")


def _newest_dep():
    deps = glob.glob(os.path.join(CSRC, "*")) + glob.glob(os.path.join(ROOT, "include", "*.h"))
    return max(os.path.getmtime(d) for d in deps)


def _compile(src, newest, verbose):
    out = os.path.join(OBJ, os.path.splitext(src)[0] + ".o")
    if os.path.exists(out) and os.path.getmtime(out) >= newest:
        return out
    cmd = [nvcc()] + ARCH + FLAGS + ["-x", "cu", "-c", os.path.join(CSRC, src), "-o", out]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return out


def build(verbose=False, jobs=None):
    """Compile every translation unit and link libestl_cuda.so; returns its path."""
    os.makedirs(OBJ, exist_ok=True)
    newest = _newest_dep()
    with cf.ThreadPoolExecutor(max_workers=jobs or min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, newest, verbose), SOURCES))
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(o) for o in objs):
        return LIB
    cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))

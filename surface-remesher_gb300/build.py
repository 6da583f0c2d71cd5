"""Build libgcvt_gb300.so (the CUDA engine and its C ABI) for sm_103a.

Usage: python build.py [--clean]
Each .cu in csrc/ is compiled in parallel with nvcc, then linked into
lib/libgcvt_gb300.so next to this file.  No CMake, no torch extension.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "lib")
OBJ = os.path.join(OUT, "obj")
LIB = os.path.join(OUT, "libgcvt_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _compile(src, extra):
    obj = os.path.join(OBJ, os.path.basename(src)[:-3] + ".o")
    cmd = [nvcc(), "-c", src, "-o", obj] + ARCH + FLAGS + extra
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(verbose=False, extra=()):
    """Compile every CUDA source and link the shared library; returns its path."""
    os.makedirs(OBJ, exist_ok=True)
    srcs = sources()
    with concurrent.futures.ThreadPoolExecutor(max_workers=max(1, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(s, list(extra)), srcs))
    objs = [o for o, _ in results]
    if verbose:
        for o, err in results:
            if err.strip():
                print(os.path.basename(o), err, file=sys.stderr)
    cmd = [nvcc(), "-shared", "-o", LIB] + objs + ARCH + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    if "--clean" in sys.argv and os.path.isdir(OUT):
        shutil.rmtree(OUT)
    print(build(verbose=True))

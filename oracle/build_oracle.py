"""Build recipe for the oracle (TEST INFRASTRUCTURE ONLY).

Outputs:
  oracle/_build/liboracle.so    -- the C restatement (gcvt_oracle.c), OpenMP
  oracle/_build/librefh.so      -- ref_harness.c, the driver-API host side that
                                   launches the reference's kernels
  oracle/_ref/gcvt_ref.cubin    -- the reference's source/gcvt.cu, compiled from
  oracle/_ref/raster_ref.cubin     its own sources in the reference checkout
                                   (only where that checkout exists; the cubins
                                   are device code and travel with the repo)
  oracle/_ref/librecover_ref.so -- ref_recover.cpp around the reference's own
                                   source/recover.h and source/weighting.h (only
                                   where the checkout exists; host code, so it
                                   does not run on another architecture)
  oracle/_ref/libseed_ref.so    -- ref_seed.cpp around the reference's own
                                   source/gcvt.h seeding (same conditions)

The reference checkout is found at $GCVT_REFERENCE_DIR, or given with
--reference DIR, or else taken to be the directory `reference` beside this
repository's root.

The reference's gcvt.cu includes <helper_timer.h> from the CUDA Samples
(gcvt.cu:27) without using it; an empty stand-in header is generated under
oracle/_ref/stub/.  Nothing from the reference is copied into the repository.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
REFERENCE = os.environ.get("GCVT_REFERENCE_DIR") or os.path.normpath(
    os.path.join(HERE, "..", "..", "reference"))
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))


def build_oracle():
    os.makedirs(BUILD, exist_ok=True)
    out = os.path.join(BUILD, "liboracle.so")
    _run(["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c11", "-Wall",
          "-ffp-contract=off", "-o", out, os.path.join(HERE, "gcvt_oracle.c"), "-lm"])
    return out


def build_harness():
    os.makedirs(BUILD, exist_ok=True)
    out = os.path.join(BUILD, "librefh.so")
    stubs = os.path.join(CUDA, "lib64", "stubs")
    _run(["gcc", "-O2", "-fPIC", "-shared", "-std=c11", "-ffp-contract=off",
          "-I", os.path.join(CUDA, "include"), "-o", out, os.path.join(HERE, "ref_harness.c"),
          "-L", stubs, "-lcuda", "-lm"])
    return out


def build_reference_cubins():
    """Compile the reference's kernels where its checkout exists; returns the
    cubin paths (existing prebuilt ones when the checkout is absent)."""
    gcvt_cu = os.path.join(REFERENCE, "source", "gcvt.cu")
    raster_cu = os.path.join(REFERENCE, "source", "discretization.cu")
    out_g = os.path.join(REF_OUT, "gcvt_ref.cubin")
    out_r = os.path.join(REF_OUT, "raster_ref.cubin")
    if os.path.exists(gcvt_cu):
        stub = os.path.join(REF_OUT, "stub")
        os.makedirs(stub, exist_ok=True)
        open(os.path.join(stub, "helper_timer.h"), "w").close()
        nvcc = os.path.join(CUDA, "bin", "nvcc")
        _run([nvcc, "-cubin", "-O3", "-I", stub, "-o", out_g, gcvt_cu] + ARCH)
        _run([nvcc, "-cubin", "-O3", "-o", out_r, raster_cu] + ARCH)
    return [p for p in (out_g, out_r) if os.path.exists(p)]


def build_reference_recover():
    """The reference's recover.h / weighting.h behind ref_recover.cpp's
    stand-ins for CGAL and Boost; None where the checkout is absent."""
    src = os.path.join(REFERENCE, "source")
    if not os.path.exists(os.path.join(src, "recover.h")):
        return None
    os.makedirs(REF_OUT, exist_ok=True)
    out = os.path.join(REF_OUT, "librecover_ref.so")
    _run(["g++", "-O2", "-fPIC", "-shared", "-std=c++17", "-ffp-contract=off", "-I", src,
          "-o", out, os.path.join(HERE, "ref_recover.cpp")])
    return out


def build_reference_seed():
    """The reference's gcvt.h seeding behind ref_seed.cpp; None where the
    checkout is absent."""
    src = os.path.join(REFERENCE, "source")
    if not os.path.exists(os.path.join(src, "gcvt.h")):
        return None
    os.makedirs(REF_OUT, exist_ok=True)
    out = os.path.join(REF_OUT, "libseed_ref.so")
    _run(["g++", "-O2", "-fPIC", "-shared", "-std=c++17", "-ffp-contract=off", "-I", src,
          "-o", out, os.path.join(HERE, "ref_seed.cpp")])
    return out


def build_all():
    paths = [build_oracle()]
    for extra in (build_reference_recover, build_reference_seed):
        rr = extra()
        if rr:
            paths.append(rr)
    try:
        paths.append(build_harness())
    except RuntimeError as e:  # no CUDA headers: the harness is optional
        print("ref harness not built:", e, file=sys.stderr)
    paths += build_reference_cubins()
    return paths


if __name__ == "__main__":
    if "--reference" in sys.argv:
        REFERENCE = sys.argv[sys.argv.index("--reference") + 1]
    if "--clean" in sys.argv:
        shutil.rmtree(BUILD, ignore_errors=True)
    for p in build_all():
        print(p)

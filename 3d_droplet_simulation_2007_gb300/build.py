"""Build recipe of ``libdsg.so``: every ``csrc/*.cu`` compiled for sm_103a.

Translation units are compiled in parallel with nvcc and linked into one
shared library in ``_build/`` next to this file.  Flags:

* ``-gencode arch=compute_103a,code=sm_103a`` -- GB300 only;
* ``--fmad=false`` and host ``-ffp-contract=off`` -- no multiply-add
  contraction, so the FP64 path rounds exactly like a non-contracting build of
  the reference and parity against the oracle is bit-level where the
  arithmetic allows;
* ``-lineinfo`` -- source correlation in profiles.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libdsg.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-I" + INCLUDE]
# Files whose kernels may contract multiply-adds (precision-relaxed paths).
# Files built with FMA contraction: the FP32 multigrid, the network, and the
# FP64 momentum/CSF glue (FP64-instruction-bound on GB300; their results stay
# within ulps of the non-contracted oracle, far inside the 1e-10 parity bar).
# The array-level FP64 kernels (mg64.cu), the VOF geometry and k-epsilon stay
# uncontracted: they are bit-identical to the oracle.
# batch.cu runs the same FP32 block bodies as mg32.cu (mg32_cells.cuh) and must
# be compiled the same way so that batched members reproduce standalone bits.
FMAD_TRUE = {"mg32.cu", "batch.cu", "nn.cu", "momentum.cu", "csf.cu"}


def nvcc():
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libdsg.so")


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps():
    return sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h")) + [__file__]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in _deps())


def _compile(src, verbose):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    flags = list(NVCC_FLAGS)
    if os.path.basename(src) in FMAD_TRUE:
        flags = [f for f in flags if f != "--fmad=false"] + ["--fmad=true"]
    cmd = [nvcc()] + ARCH + flags + ["-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
    return obj


def build(force=False, verbose=False, jobs=None):
    """Compile libdsg.so if missing or stale; return its path."""
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))

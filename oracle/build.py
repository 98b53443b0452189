"""Build recipe for the CPU oracle (test infrastructure only).

Compiles ``dsg_oracle.c`` into ``oracle/_build/libdsg_oracle.so`` with
``-O2 -ffp-contract=off`` so that no multiply-add is fused and every double
rounding follows the Fortran expression order of main.f.  The same flags are
used on x86_64 and aarch64 (aarch64 GCC contracts to FMA unless told not to).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libdsg_oracle.so")
SRC = [os.path.join(HERE, "dsg_oracle.c")]
HDR = [os.path.join(HERE, "dsg_oracle.h")]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in SRC + HDR + [__file__])


def build(force=False, verbose=False):
    """Compile the oracle shared library if it is missing or out of date."""
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-std=c11", "-fPIC", "-shared",
           "-Wall", "-o", LIB] + SRC + ["-lm"]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.check_call(cmd)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))

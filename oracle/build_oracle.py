"""Build recipe for the C oracle (test infrastructure only).

Compiles oracle/oracle.c with gcc + OpenMP into oracle/_build/liboracle.so.
Plain C, no architecture-specific flags, so the same recipe works on x86_64
and aarch64 hosts.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")


def build(force=False):
    src = [os.path.join(HERE, "oracle.c"), os.path.join(HERE, "oracle_impl.h")]
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(s) for s in src)):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-std=c99",
           "-o", tmp, src[0], "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))

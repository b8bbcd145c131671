"""Build the CUDA engine library libgauss_radon.so for sm_103a.

Each translation unit under csrc/ is compiled by nvcc in parallel and linked
into ``_build/libgauss_radon.so`` inside the package directory (in-tree, git
ignored).  The library is a plain C-ABI shared object (include/gauss_radon.h);
the Python side loads it with ctypes.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INC = os.path.join(ROOT, "include")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libgauss_radon.so")
SOURCES = ["gr_api.cu", "gr_project.cu", "gr_derivs.cu", "gr_probe.cu", "gr_noalloc.cu",
           "gr_update.cu", "gr_volume.cu", "gr_loop.cu", "gr_reg.cu",
           "gr_moments.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        p = os.path.join(cand, "bin", "nvcc") if cand else ""
        if p and os.path.exists(p):
            return p
    return "nvcc"


def _flags(verbose):
    f = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                "-I", INC, "-I", CSRC]
    if verbose:
        f += ["-Xptxas", "-v"]
    return f


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, s) for s in os.listdir(CSRC)]
    deps.append(os.path.join(INC, "gauss_radon.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    if not force and not _stale():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    exe = nvcc()

    def compile_one(src):
        obj = os.path.join(OUT, src.replace(".cu", ".o"))
        cmd = [exe] + _flags(verbose) + ["-c", os.path.join(CSRC, src), "-o", obj]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, res.stdout, res.stderr))
        return obj, res.stderr

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(compile_one, SOURCES))
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [exe] + ARCH + ["-shared", "-o", tmp] + [o for o, _ in results] + ["-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (res.stdout, res.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))

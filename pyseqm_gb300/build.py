"""Build the native library ``_build/libpyseqm_gb300.so`` for sm_103a.

Each ``csrc/*.cu`` translation unit is compiled by nvcc in parallel, then linked
into one shared library against the shared CUDA runtime (so a process that has
already loaded ``libcudart.so.13`` through PyTorch shares it).  Rebuilds only
what changed (object newer than its sources and headers).
"""

import concurrent.futures
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
LIB = os.path.join(BUILD, "libpyseqm_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def nvcc():
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the pyseqm_gb300 CUDA library cannot be built")
    return cand


def _deps():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def _compile(src, extra):
    obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
    if not _stale(obj, [src] + _deps()):
        return obj, None
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + extra + ["-I", INCLUDE, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, "compile failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr
    return obj, r.stderr if "-Xptxas" in " ".join(extra) else None


def build(verbose=False, extra=None):
    """Compile and link; returns the library path.  Raises RuntimeError on failure."""
    os.makedirs(BUILD, exist_ok=True)
    extra = list(extra or [])
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(s, extra), srcs))
    objs = []
    for obj, msg in results:
        if msg and msg.startswith("compile failed"):
            raise RuntimeError(msg)
        if msg and verbose:
            print(msg, file=sys.stderr)
        objs.append(obj)
    if _stale(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "shared", "-o", LIB] + objs + [
            "-Xlinker", "-rpath=/usr/local/cuda/lib64"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return LIB


if __name__ == "__main__":
    v = "-v" in sys.argv
    print(build(verbose=v, extra=["-Xptxas", "-v"] if v else None))

"""Build libfen_gb300.so in-tree with nvcc for sm_103a.

The library is one CUDA translation unit per arithmetic form; they compile in parallel.  The
debug library libfen_gb300_debug.so (FEN_DEBUG_CHECKS: every field index of the kernels is
bounds-checked and recorded, see fen_debug_checks in include/fen_gpu.h) is compiled from the
same sources beside it.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libfen_gb300.so")
DEBUG_LIB = os.path.join(HERE, "libfen_gb300_debug.so")
SOURCES = ["fen_api.cu", "fen_noalloc.cu", "fen_ensemble.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
         "-diag-suppress", "815"]
VARIANTS = {LIB: [], DEBUG_LIB: ["-DFEN_DEBUG_CHECKS"]}


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def _stale(lib):
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(HERE, "..", "include", "fen_gpu.h"))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force=False, verbose=False):
    """Compile the release and debug libraries (each only when stale); returns the release path."""
    nvcc = _nvcc()
    todo = [lib for lib in VARIANTS if force or _stale(lib)]
    if not todo:
        return LIB

    def run(cmd):
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        subprocess.check_call(cmd)

    cmds, objs = [], {}
    for lib in todo:
        tag = "dbg" if lib == DEBUG_LIB else "rel"
        objs[lib] = []
        for src in SOURCES:
            obj = os.path.join(CSRC, f"{os.path.splitext(src)[0]}_{tag}.o")
            objs[lib].append(obj)
            cmds.append([nvcc, *ARCH, *FLAGS, *VARIANTS[lib], "-c", os.path.join(CSRC, src), "-o", obj])
    with ThreadPoolExecutor(max_workers=max(1, len(cmds))) as ex:
        list(ex.map(run, cmds))
    for lib in todo:
        tmp = lib + ".tmp"
        run([nvcc, *ARCH, "-shared", "-o", tmp, *objs[lib]])
        os.replace(tmp, lib)
        for o in objs[lib]:
            os.remove(o)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))

"""Builds the engine's shared library in-tree: datamininglibs_gb300/libdml_gb300.so.

nvcc compiles every CUDA translation unit for sm_103a only (one -gencode), the
host C++ with -ffp-contract=off (the n*ln(n) table and every host-side float
step round exactly as the oracle's), and links one shared library exporting the
C ABI of include/dml.h.  Translation units compile in parallel.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libdml_gb300.so")

CUDA_SOURCES = ["fit.cu", "predict.cu", "server.cu", "oob.cu", "ranks.cu", "tuning.cu"] + [
    "search_cw%d.cu" % cw for cw in (1, 2, 4, 5, 8, 16)]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return path


def _compile(src, extra):
    obj = os.path.join(BUILD, os.path.splitext(os.path.basename(src))[0] + ".o")
    cmd = [nvcc(), "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC",
           "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-fvisibility=hidden",
           "--expt-relaxed-constexpr", "-I" + os.path.join(ROOT, "include"), "-I" + CSRC,
           *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    return obj, r.stderr


def build(verbose=False, extra=()):
    os.makedirs(BUILD, exist_ok=True)
    srcs = [s for s in CUDA_SOURCES if os.path.exists(os.path.join(CSRC, s))]
    with cf.ThreadPoolExecutor(max_workers=min(os.cpu_count() or 4, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(s, list(extra)), srcs))
    objs = [o for o, _ in results]
    if verbose:
        for _, err in results:
            if err:
                sys.stderr.write(err)
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-shared", *ARCH, "-o", tmp, *objs, "-lcudart", "-lpthread", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, LIB)
    build_shim()
    return LIB


SHIM_SRC = os.path.join(HERE, "shim", "src", "shim.cc")
SHIM_LIB = os.path.join(HERE, "libdml_gb300_shim.so")


def build_shim():
    """The C++ drop-in (shim/include/datamininglibs.h) over the C ABI."""
    tmp = SHIM_LIB + ".tmp"
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-Wall",
           "-I" + os.path.join(HERE, "shim", "include"), SHIM_SRC, "-o", tmp,
           "-L" + HERE, "-ldml_gb300", "-Wl,-rpath,$ORIGIN", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("shim build failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, SHIM_LIB)
    return SHIM_LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv,
                extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else []))

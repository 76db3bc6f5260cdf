"""Build libgsevt.so (the C-ABI CUDA library) for sm_103a with nvcc.

Each .cu file is compiled to an object in parallel, then linked into
gs-evt_gb300/gsevt/_build/libgsevt.so.  -fmad=false keeps every multiply and add
separately rounded unless the source writes fmaf(), which is what makes the forward
stages bit-identical to the CPU oracle.  The files in CONTRACT hold only gradient and pose
arithmetic (parity is a tolerance there) and are compiled with contraction allowed.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
REPO = os.path.dirname(PKG)
OUT_DIR = os.path.join(PKG, "gsevt", "_build")
LIB = os.path.join(OUT_DIR, "libgsevt.so")
SOURCES = ["preprocess.cu", "preprocess_cached.cu", "binning.cu", "sort.cu", "blend.cu", "loss.cu", "track.cu",
           "events.cu", "ingest.cu", "capi.cu"]
CONTRACT = {"preprocess_cached.cu", "track.cu"}
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17", "-fmad=false",
         "-Xcompiler", "-fPIC", "-I", os.path.join(REPO, "include"), "-I", HERE]


def _deps():
    files = [os.path.join(HERE, s) for s in SOURCES]
    files += [os.path.join(HERE, "common.cuh"), os.path.join(REPO, "include", "gsevt.h"), __file__]
    return max(os.path.getmtime(f) for f in files)


def build(force=False, verbose=False, extra_flags=()):
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)

    def compile_one(src):
        obj = os.path.join(OUT_DIR, src.replace(".cu", ".o"))
        flags = [("-fmad=true" if f == "-fmad=false" and src in CONTRACT else f) for f in FLAGS]
        cmd = [NVCC, *flags, *extra_flags, "-c", os.path.join(HERE, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
        if verbose and r.stderr.strip():
            print(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [NVCC, "-shared", "-gencode", "arch=compute_103a,code=sm_103a", *objs, "-o", tmp, "-lcudart", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    extra = ["-Xptxas", "-v"] if "--ptxas" in sys.argv else []
    print(build(force="--force" in sys.argv, verbose=True, extra_flags=extra))

"""Builds the GB300 (sm_103a) CUDA library in-tree:
``allscale_ipic3d_gb300/_lib/libipic3d_gb300.so``.

The FP64 particle kernels and the field kernels are compiled with
``-fmad=false``: the reference's x86 build never fuses a multiply with an
add, and the FP64 path reproduces its rounding term by term. The FP32
kernels keep fused multiply-adds.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libipic3d_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# source -> extra flags
SOURCES = {
    "ipic3d_gpu.cu": [],
    "particles_fp64.cu": ["-fmad=false"],
    # FP32 push: flush denormals, approximate division / sqrt (the error bar
    # of the FP32 path is stated against the FP64 path)
    "particles_fp32.cu": ["--ftz=true", "--prec-div=false", "--prec-sqrt=false"],
    "fields.cu": ["-fmad=false"],
    "upload.cu": ["-fmad=false"],
    "init.cu": ["-fmad=false"],
    "noalloc.cu": ["-fmad=false"],
    "tracer.cu": ["-fmad=false"],
    "contrib.cu": ["-fmad=false"],
}


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the library")
    return exe


def _sources_mtime():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files += [os.path.join(HERE, "..", "include", f) for f in ("ipic3d_gpu.h", "ipic3d_types.h")]
    files.append(os.path.abspath(__file__))
    return max(os.path.getmtime(f) for f in files)


def build(force=False, verbose=False):
    """Compiles every .cu in parallel and links the shared library. Returns
    its path. Rebuilds only when a source is newer than the library."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _sources_mtime():
        return LIB
    os.makedirs(LIBDIR, exist_ok=True)
    objdir = os.path.join(LIBDIR, "obj")
    os.makedirs(objdir, exist_ok=True)
    cc = nvcc()
    # host code: no fused multiply-add either (x86 and Arm hosts round alike)
    common = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fno-strict-aliasing",
              "-Xcompiler", "-ffp-contract=off"] + ARCH

    def compile_one(item):
        src, extra = item
        obj = os.path.join(objdir, src.replace(".cu", ".o"))
        cmd = [cc] + common + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES.items()))
    tmp = LIB + ".tmp"
    cmd = [cc, "-shared"] + ARCH + ["-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))

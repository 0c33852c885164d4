"""Build step of libfdga: compiles the sm_103a kernels and the host runtime with nvcc.

Output: fddgasolver.jl_gb300/fdgasolver/_lib/libfdga.so (in-tree, git-ignored).  The translation
units are compiled in parallel, one -gencode (sm_103a), then one shared-library link.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(PKG), "csrc")
OUT_DIR = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT_DIR, "libfdga.so")
SOURCES = ["fdga_kernels.cu", "fdga_runtime.cu", "fdga_noalloc.cu", "fdga_anderson.cu", "fdga_anderson32.cu", "fdga_krylov.cu", "fdga_k3_tc.cu", "fdga_k3_tma.cu", "fdga_k3_oz.cu", "fdga_mfrg.cu", "fdga_adjoint.cu", "fdga_interp.cu"]
HEADERS = ["fdga_device.cuh", "fdga_kernels.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: libfdga needs the CUDA toolkit to build")


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in SOURCES + HEADERS]
    deps.append(os.path.join(os.path.dirname(os.path.dirname(PKG)), "include", "fdga.h"))
    return any(os.path.getmtime(p) > t for p in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    nvcc = _nvcc()
    common = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC"]

    def compile_one(src: str) -> str:
        obj = os.path.join(OUT_DIR, src + ".o")
        cmd = [nvcc] + common + ["-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd))
        subprocess.check_call(cmd)
        return obj

    with ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    subprocess.check_call([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart", "-lpthread"])
    os.replace(tmp, LIB)
    for o in objs:
        os.remove(o)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))

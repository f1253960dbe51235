"""Build recipe of libmpxg.so (the CUDA hot path and its C ABI).

Each translation unit under csrc/ (one per SQP model, the LQ solves, the
whole-body kernels and the host ABI) is compiled for sm_103a only, in
parallel, then linked in-tree into mpx_gb300/_build/libmpxg.so.  No torch
headers are involved: the library is a plain C ABI over CUDA runtime calls,
loaded with ctypes.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libmpxg.so")
SOURCES = ["mpxg_abi.cu", "sqp_rpy12.cu", "sqp_quat13.cu", "sqp_biped12.cu", "sqp_mixed.cu", "lqr.cu", "lqr_eq.cu",
           "wb.cu", "wb_sqp.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(ROOT, "include", "mpxg.h"))
    return files


def needs_build():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(f) > t for f in _deps())


def build(force=False, verbose=False, extra_flags=()):
    """Compile libmpxg.so if any source changed; returns its path."""
    if not force and not needs_build():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    nvcc = _nvcc()
    tag = "%d" % os.getpid()
    common = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-warn-spills",
              "-I", os.path.join(ROOT, "include"), *extra_flags]

    def compile_one(src):
        obj = os.path.join(OUT_DIR, os.path.splitext(src)[0] + ".%s.o" % tag)
        cmd = common + ["-c", "-o", obj, os.path.join(CSRC, src)]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        subprocess.run(cmd, check=True)
        return obj

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp." + tag
    try:
        subprocess.run([nvcc, *ARCH, "-shared", "-o", tmp, *objs], check=True)
        os.replace(tmp, LIB)
    finally:
        for o in objs:
            if os.path.exists(o):
                os.remove(o)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True, extra_flags=sys.argv[1:]))

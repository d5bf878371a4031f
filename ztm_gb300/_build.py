"""Builds libztmgrav.so (the C ABI of include/ztm_grav.h) and the GFM shim
in-tree with nvcc for sm_103a.  Used by __graft_entry__.build() and by the
package on first import when the library is missing."""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "_lib")
OBJDIR = os.path.join(ROOT, "_build", "obj")
LIB = os.path.join(LIBDIR, "libztmgrav.so")
SHIM = os.path.join(LIBDIR, "GFM")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-ffp-contract=off"]

SOURCES = ["ztm_capi.cu", "pointmass.cu", "prism.cu", "adjoint.cu", "iface.cu", "batch.cu", "trace.cu", "density.cu", "order.cu", "pm_adjoint.cu", "lm.cu"]
HOST_SOURCES = ["invert.cpp"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    """Compile every CUDA translation unit in parallel and link the library."""
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(OBJDIR, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "ztm_grav.h"))
    jobs = []
    objs = []
    for src in SOURCES + HOST_SOURCES:
        sp = os.path.join(CSRC, src)
        op = os.path.join(OBJDIR, src.rsplit(".", 1)[0] + ".o")
        objs.append(op)
        if force or _stale(op, [sp] + headers):
            flags = NVCC_FLAGS + (["-I" + os.path.join(ROOT, "include")] if src.endswith(".cpp") else [])
            jobs.append([nvcc] + flags + ["-c", sp, "-o", op])
    if jobs:
        with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            for out in ex.map(_run, jobs):
                if verbose and out.strip():
                    print(out)
    if force or _stale(LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs)
    shim_src = os.path.join(CSRC, "gfm_shim.cpp")
    if os.path.exists(shim_src) and (force or _stale(SHIM, [shim_src, LIB])):
        _run(["g++", "-O2", "-std=c++17", "-Wall", "-o", SHIM, shim_src,
              "-I" + os.path.join(ROOT, "include"), "-L" + LIBDIR, "-lztmgrav",
              "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
    print(LIB)

"""Build recipe of the oracle (test infrastructure, never shipped):

  oracle/_build/liboracle.so   the C restatement (oracle.c), gcc, -ffp-contract=off
  oracle/_build/libref_runner.so  driver-API loader of the reference GF kernel
  oracle/_ref/gf_ref.cubin     the reference GFM_GPU.cu kernel compiled UNCHANGED
                               from the reference sources (only where they exist;
                               the GPU host reuses the image built here)
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF = os.path.join(HERE, "_ref")
LIB = os.path.join(BUILD, "liboracle.so")
RUNNER = os.path.join(BUILD, "libref_runner.so")
CUBIN = os.path.join(REF, "gf_ref.cubin")
REF_GFM = "/root/reference/GFM_GPU.cu"


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed: %s\n%s" % (" ".join(cmd), r.stdout))


def _stale(t, deps):
    return not os.path.exists(t) or any(os.path.getmtime(d) > os.path.getmtime(t) for d in deps)


def build(force=False):
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "oracle.c")
    if force or _stale(LIB, [src, os.path.join(HERE, "oracle.h")]):
        _run(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-pthread",
              "-o", LIB, src, "-lm"])
    rsrc = os.path.join(HERE, "ref_gf_runner.cpp")
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    if force or _stale(RUNNER, [rsrc]):
        try:
            _run(["g++", "-O2", "-fPIC", "-shared", "-o", RUNNER, rsrc, "-I" + cuda + "/include",
                  "-L" + cuda + "/lib64", "-L" + cuda + "/lib64/stubs", "-lcuda"])
        except RuntimeError:
            pass  # no driver stub here: the runner is only needed on a GPU host
    if os.path.exists(REF_GFM):
        os.makedirs(REF, exist_ok=True)
        wrap = os.path.join(HERE, "ref_gf.cu")
        if force or _stale(CUBIN, [wrap, REF_GFM]):
            _run(["nvcc", "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3",
                  '-DZTM_REF_GFM="%s"' % REF_GFM, "-o", CUBIN, wrap])
    return LIB


if __name__ == "__main__":
    print(build(force=True))

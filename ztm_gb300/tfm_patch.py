"""Puts this library behind ZTM's gravity forward model in place: rewrites a
copy of ZTM's TFM.cpp so that FM::FM computes the gravity field in process
through include/ztm_grav.hpp instead of the /dev/shm + popen("./GFM")
protocol.

  python -m ztm_gb300.tfm_patch path/to/TFM.cpp out/TFM.cpp

Three edits, each anchored on the reference's own text (the tool stops if an
anchor is missing or not unique):

1. after the last source include (TFM.cpp:51, `#include "SET.cpp"`):
   `#include "ztm_grav.hpp"`;
2. the GPU branch of the gravity model (TFM.cpp:90-94: float32 files, popen,
   read back) becomes one call of ztm::gfm over the same drho, surf, nn and
   G, and the CPU branch that follows (TFM.cpp:95, `else{`) becomes
   `if(!GPU){`, so that a non-zero status falls back to the unchanged CPU
   lambda in the same call;
3. the start-up step that compiles GFM_GPU.cu with nvcc and drops to the CPU
   model when that fails (TFM.cpp:207-208) becomes a check that a GPU
   context can be created.

Build the result with the reference's own command plus the library:
  g++ -o TFM TFM.cpp -lpthread -O3 -I<repo>/include -L<repo>/ztm_gb300/_lib
      -lztmgrav -Wl,-rpath,<repo>/ztm_gb300/_lib
(run from the directory holding zmath.cpp, FMM.cpp, NNI.cpp and SET.cpp, or
add -I for it).
"""
import re
import sys

INCLUDE_ANCHOR = '#include "SET.cpp"'
GPU_BRANCH_START = "if(GPU){vector<float>R32, S32, G32(di*dj);"
GPU_BRANCH_END = "for(int m=0; m<di*dj; m++){G[m]=G32[m];}}"
CPU_BRANCH = "else{thread GR[dj-2*bfr];"
COMPILE_START = 'if(GPU && grav){F=popen("nvcc -o GFM GFM_GPU.cu'
COMPILE_END = 'else{GPU=false; print("GPU error:\\n\\n"+gs+"\\nUsing CPU gravity model");}}'

GFM_CALL = ("if(GPU){if(ztm::gfm(drho, surf, G, nn, di, dj, dk, fh, fv, bfr) != 0){GPU=false;}}"
            "  //ztm_gb300: gravity field in process (include/ztm_grav.hpp); on failure the CPU"
            " lambda below runs")
CTX_CHECK = ('if(GPU && grav){if(ztm::thread_ctx()){print("\\nGPU gravity model: ztm_gb300");} '
             'else{GPU=false; print("No CUDA device for ztm_gb300: using CPU gravity model");}}'
             "  //ztm_gb300: replaces the nvcc build of GFM_GPU.cu")


class PatchError(RuntimeError):
    pass


def _one(lines, needle, what):
    hits = [i for i, l in enumerate(lines) if needle in l]
    if len(hits) != 1:
        raise PatchError("%s: expected one line containing %r, found %d" % (what, needle, len(hits)))
    return hits[0]


def patch(text):
    """The patched TFM.cpp text."""
    lines = text.split("\n")
    # 1. include the C++ layer after the reference's last source include
    i = _one(lines, INCLUDE_ANCHOR, "includes")
    lines.insert(i + 1, '#include "ztm_grav.hpp"                                                       '
                        "//ztm_gb300: in-process gravity forward model")
    # 2. the GPU branch of FM::FM
    a = _one(lines, GPU_BRANCH_START, "GPU branch")
    b = _one(lines, GPU_BRANCH_END, "GPU branch end")
    if b < a or b - a > 8:
        raise PatchError("GPU branch: unexpected layout")
    indent = re.match(r"\s*", lines[a]).group(0)
    lines[a:b + 1] = [indent + GFM_CALL]
    c = _one(lines, CPU_BRANCH, "CPU branch")
    if c != a + 1:
        raise PatchError("CPU branch does not follow the GPU branch")
    lines[c] = lines[c].replace("else{thread GR[", "if(!GPU){thread GR[", 1)
    # 3. the nvcc build of GFM_GPU.cu at start-up
    s = _one(lines, COMPILE_START, "GFM build")
    e = _one(lines, COMPILE_END, "GFM build end")
    if e != s + 1:
        raise PatchError("GFM build: unexpected layout")
    indent = re.match(r"\s*", lines[s]).group(0)
    lines[s:e + 1] = [indent + CTX_CHECK]
    return "\n".join(lines)


def main(argv):
    if len(argv) != 3:
        print(__doc__)
        return 2
    with open(argv[1], encoding="latin-1") as f:
        text = f.read()
    out = patch(text)
    with open(argv[2], "w", encoding="latin-1") as f:
        f.write(out)
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))

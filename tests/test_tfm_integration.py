"""ZTM-side integration: the in-process patch of TFM.cpp (ztm_gb300/tfm_patch)
applied to a copy of the reference's TFM.cpp builds and links against
libztmgrav.so (TFM itself cannot run here: its data files are absent), and a
C++ program that calls ztm::gfm of include/ztm_grav.hpp with TFM-shaped
std::vector inputs matches the reference's own CPU lambda on the GPU."""
import os
import shutil
import subprocess

import pytest

import oracle
from oracle.build import REF_DIR
from ztm_gb300 import _build, tfm_patch

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")


def _have_ref():
    return os.path.exists(os.path.join(REF_DIR, "TFM.cpp"))


@pytest.mark.skipif(not _have_ref(), reason="reference TFM.cpp not present")
def test_patch_anchors_and_edits():
    src = open(os.path.join(REF_DIR, "TFM.cpp"), encoding="latin-1").read()
    out = tfm_patch.patch(src)
    assert '#include "ztm_grav.hpp"' in out
    assert "ztm::gfm(drho, surf, G, nn, di, dj, dk, fh, fv, bfr)" in out
    assert 'popen("./GFM"' not in out and "nvcc -o GFM" not in out
    assert "if(!GPU){thread GR[dj-2*bfr];" in out
    # the CPU lambda itself is untouched
    lam = [l for l in src.split("\n") if "auto GFM=[&](int j0)" in l]
    assert len(lam) == 1 and lam[0] in out
    with pytest.raises(tfm_patch.PatchError):
        tfm_patch.patch(out)  # anchors gone: a second application is refused


@pytest.mark.skipif(not _have_ref(), reason="reference TFM.cpp not present")
def test_patched_tfm_compiles_and_links(tmp_path):
    src = open(os.path.join(REF_DIR, "TFM.cpp"), encoding="latin-1").read()
    p = tmp_path / "TFM.cpp"
    p.write_text(tfm_patch.patch(src), encoding="latin-1")
    libdir = os.path.dirname(_build.LIB)
    r = subprocess.run(["g++", "-std=c++14", "-O1", "-o", str(tmp_path / "TFM"), str(p),
                        "-I" + INCLUDE, "-I" + REF_DIR, "-lpthread", "-L" + libdir, "-lztmgrav",
                        "-Wl,-rpath," + libdir], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    assert os.path.exists(tmp_path / "TFM")


@pytest.mark.gpu
@pytest.mark.skipif(not oracle.ref_tfm_available(), reason="reference TFM.cpp lambda not built")
def test_cpp_header_on_gpu_matches_reference_lambda(tmp_path):
    from oracle import build as ob
    libdir = os.path.dirname(_build.LIB)
    exe = tmp_path / "gfm_hpp_check"
    r = subprocess.run(["g++", "-std=c++14", "-O2", "-o", str(exe),
                        os.path.join(ROOT, "tests", "cpp", "gfm_hpp_check.cpp"), "-I" + INCLUDE,
                        "-L" + libdir, "-lztmgrav", os.path.abspath(ob.TFM_LIB), "-lpthread",
                        "-Wl,-rpath," + libdir + ":" + os.path.dirname(os.path.abspath(ob.TFM_LIB))],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-3000:]
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stdout + run.stderr
    assert "normwise rel err" in run.stdout

"""Build recipe of the oracle (test infrastructure, never shipped):

  oracle/_build/liboracle.so   the C restatement (oracle.c), gcc, -ffp-contract=off
  oracle/_build/libref_runner.so  driver-API loader of the reference GF kernel
  oracle/_ref/gf_ref.cubin     the reference GFM_GPU.cu kernel compiled UNCHANGED
                               from the reference sources
  oracle/_ref/tfm_gfm.cpp      the reference's CPU gravity lambda (TFM.cpp:95-99)
                               cut VERBATIM out of TFM.cpp into a small C
                               harness (generated, never committed)
  oracle/_ref/libref_tfm.so    that harness compiled with g++
  oracle/_ref/zmath_lm.cpp     the reference's zmath.cpp VERBATIM, followed by a
                               harness around the damped Gauss-Newton step of
                               LMA::fit (TFM.cpp:159-160, cut verbatim)
  oracle/_ref/libref_lm.so     that file compiled with g++

The reference directory is ZTM_REFERENCE_DIR (default: the read-only copy
this repository was built beside).  Where it is absent (the GPU host), the
generated harness source that travels in oracle/_ref/ is compiled there; the
cubin is GPU code and is used as it is.
"""
import os
import re
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF = os.path.join(HERE, "_ref")
LIB = os.path.join(BUILD, "liboracle.so")
RUNNER = os.path.join(BUILD, "libref_runner.so")
CUBIN = os.path.join(REF, "gf_ref.cubin")
TFM_SRC = os.path.join(REF, "tfm_gfm.cpp")
TFM_LIB = os.path.join(REF, "libref_tfm.so")
LM_SRC = os.path.join(REF, "zmath_lm.cpp")
LM_LIB = os.path.join(REF, "libref_lm.so")
REF_DIR = os.environ.get("ZTM_REFERENCE_DIR", "/root/reference")
REF_GFM = os.path.join(REF_DIR, "GFM_GPU.cu")
REF_TFM = os.path.join(REF_DIR, "TFM.cpp")
REF_ZMATH = os.path.join(REF_DIR, "zmath.cpp")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed: %s\n%s" % (" ".join(cmd), r.stdout))


def _stale(t, deps):
    return not os.path.exists(t) or any(os.path.getmtime(d) > os.path.getmtime(t) for d in deps)


# The harness around the reference lambda.  The lambda captures by reference
# exactly the names FM::FM has in scope at TFM.cpp:95 (di, dj, bfr, ii, jj, fh,
# fv, surf, G, nn, drho; zmath.cpp:19-21 supplies vec, ivec and thread), so the
# harness declares those and nothing else.
_HARNESS_HEAD = """\
// GENERATED by oracle/build.py from the reference's TFM.cpp -- not committed.
// The lines marked VERBATIM are copied unchanged from TFM.cpp (line numbers
// in the markers); everything else is the harness that gives them their
// scope.  Test and baseline infrastructure only.
#include <math.h>
#include <thread>
#include <vector>
typedef std::vector<double> vec;  // zmath.cpp:19
typedef std::vector<int> ivec;    // zmath.cpp:19
using std::thread;                // zmath.cpp:21

// G (di*dj) from drho (N fine-grid nodes), nn (n_nn indices) and surf (di*dj),
// through TFM.cpp:95-99 as written: one std::thread per interior station row.
extern "C" void ref_tfm_gfm(int di, int dj, int dk, int fh, int fv, int bfr, const double* drho_p,
                            long long N, const int* nn_p, long long n_nn, const double* surf_p,
                            double* G_p) {
  int ii = (di - 1) * fh + 1, jj = (dj - 1) * fh + 1;  // TFM.cpp:83
  (void)dk;
  vec drho(drho_p, drho_p + N), surf(surf_p, surf_p + (long long)di * dj);
  vec G(G_p, G_p + (long long)di * dj);
  ivec nn(nn_p, nn_p + n_nn);
"""

_HARNESS_ROWS = """\
  for (long long m = 0; m < (long long)di * dj; m++) G_p[m] = G[m];
}

// The same lambda for the interior rows j0 in [row_lo, row_hi) only, one
// std::thread per row (the reference's own threading): a bounded sample of
// the full call for timing.  Rows outside the range are left as passed in.
extern "C" void ref_tfm_gfm_rows(int di, int dj, int dk, int fh, int fv, int bfr,
                                 const double* drho_p, long long N, const int* nn_p,
                                 long long n_nn, const double* surf_p, double* G_p, int row_lo,
                                 int row_hi) {
  int ii = (di - 1) * fh + 1, jj = (dj - 1) * fh + 1;  // TFM.cpp:83
  (void)dk;
  vec drho(drho_p, drho_p + N), surf(surf_p, surf_p + (long long)di * dj);
  vec G(G_p, G_p + (long long)di * dj);
  ivec nn(nn_p, nn_p + n_nn);
"""

_HARNESS_TAIL = """\
  std::vector<thread> rows;
  for (int j0 = row_lo; j0 < row_hi; j0++)
    if (j0 >= bfr && j0 < dj - bfr) rows.emplace_back(GFM, j0);
  for (auto& t : rows) t.join();
  for (long long m = 0; m < (long long)di * dj; m++) G_p[m] = G[m];
}
"""


def extract_tfm_lambda(tfm_path=REF_TFM):
    """The CPU gravity branch of FM::FM (TFM.cpp:95-99), verbatim: the thread
    array, the three lines of the GFM lambda, and the launch/join line.
    Returns (thread_decl, lambda_lines, launch, first_line_number)."""
    lines = open(tfm_path, encoding="latin-1").read().split("\n")
    start = next(i for i, l in enumerate(lines) if "auto GFM=[&](int j0)" in l)
    end = next(i for i in range(start, len(lines)) if "}}};" in lines[i])
    lam = [lines[i].strip() for i in range(start, end + 1)]
    decl_line = lines[start - 1]
    m = re.search(r"thread GR\[dj-2\*bfr\];", decl_line)
    if not m:
        raise RuntimeError("TFM.cpp: no thread array before the GFM lambda")
    launch_line = lines[end + 1]
    m2 = re.search(r"for\(int j=0;j<dj-2\*bfr;j\+\+\)\{GR\[j\]=thread\(GFM,j\+bfr\);\} "
                   r"for\(auto&w:GR\)\{w\.join\(\);\}", launch_line)
    if not m2:
        raise RuntimeError("TFM.cpp: no launch line after the GFM lambda")
    return m.group(0), lam, m2.group(0), start + 1


def write_tfm_harness(tfm_path=REF_TFM, out=TFM_SRC):
    decl, lam, launch, first = extract_tfm_lambda(tfm_path)
    n0, n1 = first - 1, first + len(lam)
    body = ["  // VERBATIM TFM.cpp:%d (from 'thread GR')" % n0, "  " + decl]
    body.append("  // VERBATIM TFM.cpp:%d-%d" % (first, first + len(lam) - 1))
    body += ["  " + l for l in lam]
    body += ["  // VERBATIM TFM.cpp:%d (up to the join)" % n1, "  " + launch]
    rows = ["  // VERBATIM TFM.cpp:%d-%d" % (first, first + len(lam) - 1)] + ["  " + l for l in lam]
    src = (_HARNESS_HEAD + "\n".join(body) + "\n" + _HARNESS_ROWS + "\n".join(rows) + "\n" +
           _HARNESS_TAIL)
    os.makedirs(os.path.dirname(out), exist_ok=True)
    with open(out, "w") as f:
        f.write(src)
    return out


_LM_HARNESS = """
// ---- harness (GENERATED by oracle/build.py; not part of zmath.cpp) --------
// The damped Gauss-Newton step of LMA::fit, TFM.cpp:159-160 (the two
// statements marked VERBATIM), for a given Jacobian J (nrows x ncols,
// J[data][parameter]), residual r = y - f, parameters b, uncertainties sig
// and nd damping pairs dm: B[n] = b + inv(JJ + d0 M + d1 A) J^T r.
struct ZtmLmArgs {
  vec sig;
};
extern "C" void ref_lm_steps(const double* Jp, int nrows, int ncols, const double* rp,
                             const double* bp, const double* sigp, const double* dmp, int nd,
                             double* Bout, double* JJout) {
  mat J(nrows, vec(ncols)), JJ, M, A;
  for (int i = 0; i < nrows; i++)
    for (int j = 0; j < ncols; j++) J[i][j] = Jp[(long long)i * ncols + j];
  vec r(rp, rp + nrows), b(bp, bp + ncols);
  ZtmLmArgs S;
  S.sig = vec(sigp, sigp + ncols);
  mat B(nd);
  // VERBATIM TFM.cpp:159 (from 'JJ=MTM(J)')
  %(line159)s
  // VERBATIM TFM.cpp:160
  %(line160)s
  for (int n = 0; n < nd; n++) F(n, vec{dmp[2 * n], dmp[2 * n + 1]});
  for (int n = 0; n < nd; n++)
    for (int j = 0; j < ncols; j++) Bout[(long long)n * ncols + j] = B[n][j];
  if (JJout)
    for (int i = 0; i < ncols; i++)
      for (int j = 0; j < ncols; j++) JJout[(long long)i * ncols + j] = JJ[i][j];
}
"""


def write_lm_harness(zmath_path=REF_ZMATH, tfm_path=REF_TFM, out=LM_SRC):
    """zmath.cpp verbatim + the LMA step of TFM.cpp:159-160."""
    zm = open(zmath_path, encoding="latin-1").read()
    lines = open(tfm_path, encoding="latin-1").read().split("\n")
    i = next(k for k, l in enumerate(lines) if "JJ=MTM(J); M=diag(diag(JJ)); A=diag(1/(S.sig^2));" in l)
    m = re.search(r"JJ=MTM\(J\); M=diag\(diag\(JJ\)\); A=diag\(1/\(S\.sig\^2\)\);", lines[i])
    m2 = re.search(r"auto F=\[&\]\(int n,vec d\)\{B\[n\]=b\+inv\(JJ\+d\[0\]\*M\+d\[1\]\*A\)\*T\(J\)\*r;\};",
                   lines[i + 1])
    if not m or not m2:
        raise RuntimeError("TFM.cpp: LMA step lines not found")
    src = ("// GENERATED by oracle/build.py: the reference's zmath.cpp, unchanged, then a\n"
           "// harness.  Test and baseline infrastructure only; never committed.\n" + zm +
           _LM_HARNESS % {"line159": m.group(0), "line160": m2.group(0)})
    os.makedirs(os.path.dirname(out), exist_ok=True)
    with open(out, "w", encoding="latin-1") as f:
        f.write(src)
    return out


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
    if os.path.exists(REF_TFM) and (force or _stale(TFM_SRC, [REF_TFM, __file__])):
        write_tfm_harness()
    if os.path.exists(TFM_SRC) and (force or _stale(TFM_LIB, [TFM_SRC])):
        # the reference builds with g++ -O3 (TFM.cpp:11); contraction is
        # switched off so that x86 and Arm hosts round alike
        _run(["g++", "-O3", "-std=c++14", "-ffp-contract=off", "-fPIC", "-shared", "-pthread",
              "-o", TFM_LIB, TFM_SRC])
    if os.path.exists(REF_ZMATH) and os.path.exists(REF_TFM) and (
            force or _stale(LM_SRC, [REF_ZMATH, REF_TFM, __file__])):
        write_lm_harness()
    if os.path.exists(LM_SRC) and (force or _stale(LM_LIB, [LM_SRC])):
        _run(["g++", "-O3", "-std=c++14", "-ffp-contract=off", "-fPIC", "-shared", "-pthread",
              "-w", "-o", LM_LIB, LM_SRC])
    return LIB


if __name__ == "__main__":
    print(build(force=True))

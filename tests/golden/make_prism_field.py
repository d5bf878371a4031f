"""Makes tests/golden/prism_256x256x64_draped_fp64.npz: the double-precision
field of the 256x256x64 draped prism mesh (1 x 1 x 0.5 km cells) at all
128 x 128 stations, from the CPU oracle (oracle/oracle.c: the closed-form
8-corner prism sum in double, every prism at every station), so that the
GPU's mixed and plain-double forwards can be checked on the whole field
rather than on a station subset.

The inputs are regenerated from their seed (ztm_gb300.synth), so the fixture
holds only the field and fingerprints of the inputs it was computed from
(sums and a strided sample of the densities, the station coordinates' sums),
which the tests compare before they use it.

  python tests/golden/make_prism_field.py [--threads N]

About 35 minutes on 8 x86 cores.
"""
import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
OUT = os.path.join(HERE, "prism_256x256x64_draped_fp64.npz")


def fingerprint(rho, st):
    return {"rho_sum": float(np.sum(rho)), "rho_abs_sum": float(np.sum(np.abs(rho))),
            "rho_sample": np.asarray(rho[::9973], dtype=np.float64),
            "st_sum": np.sum(st, axis=0).astype(np.float64)}


def main():
    import oracle
    from ztm_gb300 import synth
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--chunk", type=int, default=1024)
    args = ap.parse_args()
    mesh, rho, st = synth.draped_mesh_256x256x64()
    gz = np.empty(len(st))
    t0 = time.time()
    for a in range(0, len(st), args.chunk):
        b = min(len(st), a + args.chunk)
        gz[a:b] = oracle.prism_mesh(mesh, rho, st[a:b], nthreads=args.threads)
        print("%5d / %d stations, %.0f s" % (b, len(st), time.time() - t0), flush=True)
    fp = fingerprint(rho, st)
    np.savez_compressed(OUT, gz=gz, G=np.float64(6.67e-11), **fp)
    print("wrote", OUT)


if __name__ == "__main__":
    main()

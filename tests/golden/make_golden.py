"""Generates tests/golden/gf_*.npz: outputs of the reference GF kernel
(GFM_GPU.cu:16-22, compiled unchanged into oracle/_ref/gf_ref.cubin) on
seeded point-mass inputs.  Needs a GPU and the reference image; run as
    python tests/golden/make_golden.py [outdir]
The committed fixtures were made this way."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, os.path.dirname(HERE))

import oracle  # noqa: E402
import ztm_gb300  # noqa: E402
from helpers import tfm_like_inputs  # noqa: E402

CASES = [  # di, dj, dk, fh, fv, bfr, seed
    (61, 61, 33, 1, 2, 10, 101),  # the reference's own dimensions (TFM.cpp:190)
    (31, 29, 17, 1, 2, 5, 102),
    (16, 16, 9, 1, 3, 0, 103),
]


def main(outdir):
    os.makedirs(outdir, exist_ok=True)
    for di, dj, dk, fh, fv, bfr, seed in CASES:
        g = ztm_gb300.make_grid(di, dj, dk, fh, fv, bfr)
        drho, surf = tfm_like_inputs(di, dj, dk, fh, fv, seed=seed)
        r32 = drho.astype(np.float32)
        s32 = surf.astype(np.float32)
        out, _ = oracle.ref_gf(g, r32, s32)
        name = os.path.join(outdir, "gf_%dx%dx%d_fh%d_fv%d_b%d.npz" % (di, dj, dk, fh, fv, bfr))
        np.savez_compressed(name, dims=np.array([di, dj, dk, fh, fv, bfr]), drho=r32, surf=s32,
                            g=out)
        print(name)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else HERE)

"""The far-field expansion's coefficients as shipped in
ztm_gb300/csrc/prism_common.cuh (far_coef) against their symbolic derivation
(ztm_gb300/far_expansion.py, sympy): every coefficient of orders 2, 4 and 6,
evaluated at a few cell shapes."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def shipped_coefficients():
    src = open(os.path.join(ROOT, "ztm_gb300", "csrc", "prism_common.cuh")).read()
    body = src[src.index("inline FarCoef far_coef("):]
    body = body[:body.index("return f;")]
    out = {}
    for m in re.finditer(r"f\.(\w+)\s*=\s*\(float\)\((.*?)\);", body, re.S):
        out[m.group(1)] = " ".join(m.group(2).split())
    return out


def test_far_coef_matches_the_symbolic_expansion():
    sp = pytest.importorskip("sympy")
    from ztm_gb300 import far_expansion
    shipped = shipped_coefficients()
    assert len(shipped) == 19, sorted(shipped)
    derived = far_expansion.orders(6)
    dx, dy, dz = sp.symbols("dx dy dz", positive=True)
    for cell in ((1.0, 1.0, 0.5), (1.0, 0.8, 0.5), (0.7, 1.0, 1.0), (1.0, 0.35, 0.9)):
        x2, y2, z2 = cell[0] ** 2, cell[1] ** 2, cell[2] ** 2
        env = {"x2": x2, "y2": y2, "z2": z2, "x4": x2 * x2, "y4": y2 * y2, "z4": z2 * z2,
               "x6": x2 ** 3, "y6": y2 ** 3, "z6": z2 ** 3}
        for order, names in far_expansion.NAMES.items():
            for key, name in names.items():
                want = float(derived[order][key].subs({dx: cell[0], dy: cell[1], dz: cell[2]}))
                got = eval(shipped[name], {}, env)
                assert abs(got - want) <= 1e-12 * max(1.0, abs(want)), (name, cell, got, want)

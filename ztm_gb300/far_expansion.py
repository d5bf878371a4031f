"""Derivation of the far-field expansion used by the mixed prism kernels
(ztm_gb300/csrc/prism_common.cuh: far_coef, col_poly, far_unit2).

The attraction kernel of a point mass, Z / r^3 (Z the station's height over
the mass, r the distance), averaged over a prism of edges dx, dy, dz centred
at the mass point, expanded in the prism's moments: for each order 2p the
sum over even multi-indices (i, j, k), i + j + k = 2p, of the derivative
d^(i+j+k)/dX^i dY^j dZ^k (Z/r^3) times the box averages
(dx/2)^i/(i+1) (dy/2)^j/(j+1) (dz/2)^k/(k+1) over i! j! k!.  Each order
divided by Z/r^3 is a homogeneous polynomial in X^2, Y^2, Z^2 over r^(4p);
the coefficients printed here are those of far_coef.

  python -m ztm_gb300.far_expansion            # the coefficients, C++ form
  python -m ztm_gb300.far_expansion --check    # truncation error vs q

sympy is needed for the derivation (numpy alone for --check, which uses a
closed-form prism integral written here)."""
import argparse
import math


def orders(max_order=6):
    import sympy as sp
    X, Y, Z = sp.symbols("X Y Z")
    dx, dy, dz = sp.symbols("dx dy dz", positive=True)
    f = Z / (X ** 2 + Y ** 2 + Z ** 2) ** sp.Rational(3, 2)

    def mom(h, n):
        return 0 if n % 2 else h ** n / (n + 1)

    out = {}
    for order in range(2, max_order + 1, 2):
        tot = 0
        for i in range(0, order + 1, 2):
            for j in range(0, order + 1 - i, 2):
                k = order - i - j
                d = sp.diff(f, X, i, Y, j, Z, k)
                tot += d * mom(dx / 2, i) * mom(dy / 2, j) * mom(dz / 2, k) / (
                    math.factorial(i) * math.factorial(j) * math.factorial(k))
        t = sp.together(sp.simplify(tot / f))
        num, den = sp.fraction(t)
        scale = den.subs({X: 0, Y: 0, Z: 1})
        poly = sp.Poly(sp.expand(num), X, Y, Z)
        out[order] = {(a // 2, b // 2, c // 2): sp.factor(cf / scale)
                      for (a, b, c), cf in poly.terms()}
    return out


NAMES = {2: {(1, 0, 0): "cA", (0, 1, 0): "cB", (0, 0, 1): "a1"},
         4: {(0, 0, 2): "h2", (1, 0, 1): "cX1", (0, 1, 1): "cY1", (2, 0, 0): "cXX",
             (1, 1, 0): "cXY", (0, 2, 0): "cYY"},
         6: {(0, 0, 3): "k3", (1, 0, 2): "kX2", (0, 1, 2): "kY2", (2, 0, 1): "kXX",
             (1, 1, 1): "kXY", (0, 2, 1): "kYY", (3, 0, 0): "kX3", (2, 1, 0): "kX2Y",
             (1, 2, 0): "kXY2", (0, 3, 0): "kY3"}}


def check():
    """Worst truncation error of the 4th- and 6th-order forms against the
    closed-form prism integral, relative to V/r^2, for 1 x 1 x 0.5 cells."""
    import numpy as np
    import sympy as sp
    X, Y, Z = sp.symbols("X Y Z")
    dx, dy, dz = sp.symbols("dx dy dz", positive=True)
    co = orders(6)
    cell = {dx: 1.0, dy: 1.0, dz: 0.5}
    terms = {}
    for o, d in co.items():
        e = sum(float(c.subs(cell)) * X ** (2 * a) * Y ** (2 * b) * Z ** (2 * cc)
                for (a, b, cc), c in d.items()) / (X ** 2 + Y ** 2 + Z ** 2) ** o
        terms[o] = sp.lambdify((X, Y, Z), e, "numpy")
    A, B, C = 0.5, 0.5, 0.25

    def phi(x, y, z):
        r = np.sqrt(x * x + y * y + z * z)
        return x * np.log(y + r) + y * np.log(x + r) - z * np.arctan(x * y / (z * r))

    hd = math.sqrt(A * A + B * B + C * C)
    rng = np.random.default_rng(1)
    for q in (3.0, 4.0, 5.0, 6.0, 8.0):
        d = rng.normal(size=(20000, 3))
        d /= np.linalg.norm(d, axis=1)[:, None]
        P = d * q * hd
        ex = 0.0
        for ux, sx in ((-A, -1), (A, 1)):
            for uy, sy in ((-B, -1), (B, 1)):
                for uz, sz in ((-C, -1), (C, 1)):
                    ex = ex + sx * sy * sz * phi(ux - P[:, 0], uy - P[:, 1], uz - P[:, 2])
        r = np.linalg.norm(P, axis=1)
        mono = 8 * A * B * C * P[:, 2] / r ** 3
        scale = 8 * A * B * C / r ** 2
        t = [terms[o](P[:, 0], P[:, 1], P[:, 2]) for o in (2, 4, 6)]
        e4 = np.abs(mono * (1 + t[0] + t[1]) - ex) / scale
        e6 = np.abs(mono * (1 + t[0] + t[1] + t[2]) - ex) / scale
        print("q %4.1f   fourth order %.2e   sixth order %.2e" % (q, e4.max(), e6.max()))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--check", action="store_true")
    args = ap.parse_args()
    if args.check:
        check()
        return
    import sympy as sp
    x2, y2, z2 = sp.symbols("x2 y2 z2")
    dx, dy, dz = sp.symbols("dx dy dz", positive=True)
    for o, d in orders(6).items():
        for key, name in NAMES[o].items():
            e = sp.expand(d[key].subs({dx: sp.sqrt(x2), dy: sp.sqrt(y2), dz: sp.sqrt(z2)}))
            num, den = sp.fraction(sp.together(e))
            print("  f.%s = (%s) / %s;" % (name, sp.ccode(sp.expand(num)), sp.ccode(den)))


if __name__ == "__main__":
    main()

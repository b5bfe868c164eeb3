"""Derive the 13-point, degree-7 symmetric triangle rule to full double precision.

The reference's triangle rules stop at 7 points / degree 5 (include/integrator.hpp:55-113).
The Galerkin configuration asks for a 13-point rule, so this script restates the published
degree-7 rule of Cowper (1973) / Dunavant (1985): one centroid point, two 3-point orbits
(a, a, 1-2a) and one 6-point orbit (a, b, 1-a-b).  The rounded published values are used only
as the starting guess; Newton iteration on the eight S3-invariant moment equations of degree
<= 7 (mpmath, 50 digits) fixes every digit, so the printed constants integrate every
polynomial of degree <= 7 over the triangle exactly up to double rounding.

Weights are normalised to sum to 1 (the reference multiplies by the triangle area afterwards).
Run:  python oracle/gen_tri13.py   -> prints C initialisers used by the oracle and the library.
"""
import itertools

import mpmath as mp

mp.mp.dps = 50

# published (rounded) starting values
W0, A1, W1, A2, W2, A3, B3, W3 = (
    -0.149570044467682, 0.260345966079040, 0.175615257433208, 0.065130102902216,
    0.053347235608838, 0.048690315425316, 0.312865496004874, 0.077113760890257)


def points(p):
    w0, a1, w1, a2, w2, a3, b3, w3 = p
    pts = [((mp.mpf(1) / 3, mp.mpf(1) / 3, mp.mpf(1) / 3), w0)]
    for a, w in ((a1, w1), (a2, w2)):
        c = 1 - 2 * a
        pts += [((c, a, a), w), ((a, c, a), w), ((a, a, c), w)]
    c3 = 1 - a3 - b3
    for perm in sorted(set(itertools.permutations((0, 1, 2)))):
        t = (a3, b3, c3)
        pts.append(((t[perm[0]], t[perm[1]], t[perm[2]]), w3))
    return pts


def exact_monomial(i, j):
    # integral over reference triangle (0,0),(1,0),(0,1) of x^i y^j, normalised by its area 1/2
    return 2 * mp.factorial(i) * mp.factorial(j) / mp.factorial(i + j + 2)


# eight independent moments (degree 0,2,3,4,5,6,6,7 invariants) via monomials in (l1, l2)
MONOMIALS = [(0, 0), (2, 0), (3, 0), (4, 0), (5, 0), (6, 0), (4, 2), (7, 0)]


def residual(p):
    pts = points(p)
    res = []
    for (i, j) in MONOMIALS:
        s = mp.fsum(w * (bc[1] ** i) * (bc[2] ** j) for bc, w in pts)
        res.append(s - exact_monomial(i, j))
    return res


def main():
    p = [mp.mpf(x) for x in (W0, A1, W1, A2, W2, A3, B3, W3)]
    sol = mp.findroot(lambda *q: residual(list(q)), p, tol=mp.mpf(10) ** -45)
    sol = [sol[k] for k in range(8)]
    pts = points(sol)
    # check every monomial of degree <= 7
    worst = mp.mpf(0)
    for i in range(8):
        for j in range(8 - i):
            s = mp.fsum(w * (bc[1] ** i) * (bc[2] ** j) for bc, w in pts)
            worst = max(worst, abs(s - exact_monomial(i, j)))
    assert worst < mp.mpf(10) ** -40, worst
    # stable ordering: centroid, orbit a1, orbit a2, 6-orbit sorted
    print("/* 13-point degree-7 rule: {l0, l1, l2, weight}, weights sum to 1 */")
    for bc, w in pts:
        print("    {%s, %s, %s, %s}," % tuple(mp.nstr(v, 20, min_fixed=-1, max_fixed=1) for v in (*bc, w)))


if __name__ == "__main__":
    main()

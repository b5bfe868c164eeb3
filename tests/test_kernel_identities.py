"""The device kernels evaluate an algebraically exact rearrangement of the reference's Green's
functions (see surfaceonlydeformables_gb300/csrc/sod_device.cuh).  Check, in 40-digit arithmetic,
that the rearranged G, H, B_trans and B_angular equal the literal formulas of
src/elastodynamics_cqbem_{G,H,B_trans,B_angular}_collocation.cu."""
import numpy as np
import pytest

mp = pytest.importorskip("mpmath")


def literal(r, s, rh, n, c1, c2, rho):
    kd = lambda i, j: 1 if i == j else 0
    e1, e2 = mp.exp(-r * s / c1), mp.exp(-r * s / c2)
    X = ((s * r / c1 + 1) / (s * s)) * e1 - ((s * r / c2 + 1) / (s * s)) * e2
    rn = sum(rh[k] * n[k] for k in range(3))
    U = [[(1 / (4 * mp.pi) / rho) * (((3 * rh[i] * rh[j] - kd(i, j)) / (r * r)) * X + rh[i] * rh[j] *
          (e1 / c1 ** 2 - e2 / c2 ** 2) + kd(i, j) / c2 ** 2 * e2) / r for j in range(3)] for i in range(3)]
    rs = r * s
    P = [[1 / (4 * mp.pi) * ((6 * c2 * c2 / (r * r)) * (rh[i] * n[j] + rh[j] * n[i] + (kd(i, j) - 5 * rh[i] * rh[j]) * rn)
                             * ((e1 / rs) * (1 / c1 + 1 / rs) - (e2 / rs) * (1 / c2 + 1 / rs))
                             + (e1 / (r * r)) * (2 * c2 * c2 / (c1 * c1) * (2 * rh[i] * n[j] + rh[j] * n[i]
                                                 - (6 * rh[i] * rh[j] - kd(i, j)) * rn) - rh[i] * n[j])
                             + (e2 / (r * r)) * (12 * rh[i] * rh[j] * rn - 2 * rh[i] * n[j] - 3 * rh[j] * n[i]
                                                 - 3 * kd(i, j) * rn)
                             - (e1 * s / (r * c1)) * (rh[i] * n[j] + 2 * c2 * c2 / (c1 * c1) * (rh[i] * rh[j] * rn - rh[i] * n[j]))
                             + (e2 * s / (r * c2)) * (2 * rh[i] * rh[j] * rn - kd(i, j) * rn - rh[j] * n[i]))
          for j in range(3)] for i in range(3)]
    X2, X1 = ((s * r / c2 + 1) / (s * s)) * e2, ((s * r / c1 + 1) / (s * s)) * e1
    Bt = [[-1 / (4 * mp.pi) * (((rh[i] * n[j] + rh[j] * n[i]) / (2 * r)) * (X2 - X1) + kd(i, j) * rn / r * (1 / (s * s) - X2)) / r
           for j in range(3)] for i in range(3)]
    Ba = [[[-1 / (4 * mp.pi) * ((rh[i] * rh[k] * n[j] + rh[j] * rh[k] * n[i] + kd(j, k) * n[i] + kd(i, k) * n[j]) / 2 * (X2 - X1)
                                - r * (kd(j, k) * n[i] + kd(i, k) * n[j]) / (2 * s) * (e2 / c2 - e1 / c1)
                                - r * (kd(i, j) * n[k]) / (c2 * s) * e2) / r for k in range(3)] for j in range(3)] for i in range(3)]
    return U, P, Bt, Ba


def stable(r, s, rh, n, c1, c2, rho):
    kd = lambda i, j: 1 if i == j else 0
    psi = lambda z: ((1 + z) * mp.exp(-z) - 1) / (z * z)
    z1, z2 = r * s / c1, r * s / c2
    e1, e2 = mp.exp(-z1), mp.exp(-z2)
    Y = psi(z1) / c1 ** 2 - psi(z2) / c2 ** 2
    kap = c2 ** 2 / c1 ** 2
    rn = sum(rh[k] * n[k] for k in range(3))
    al = (3 * Y + e1 / c1 ** 2 - e2 / c2 ** 2) / (4 * mp.pi * rho * r)
    be = (e2 / c2 ** 2 - Y) / (4 * mp.pi * rho * r)
    U = [[al * rh[i] * rh[j] + be * kd(i, j) for j in range(3)] for i in range(3)]
    a = 6 * c2 ** 2 * Y + (4 * kap - 1) * e1 - 2 * e2 - (1 - 2 * kap) * z1 * e1
    b = 6 * c2 ** 2 * Y + 2 * kap * e1 - 3 * e2 - z2 * e2
    d = -30 * c2 ** 2 * Y - 12 * kap * e1 + 12 * e2 - 2 * kap * z1 * e1 + 2 * z2 * e2
    P = [[(a * rh[i] * n[j] + b * (n[i] * rh[j] + rn * kd(i, j)) + d * rn * rh[i] * rh[j]) / (4 * mp.pi * r * r)
          for j in range(3)] for i in range(3)]
    Bt = [[((Y / 2) * (rh[i] * n[j] + rh[j] * n[i]) + psi(z2) / c2 ** 2 * rn * kd(i, j)) / (4 * mp.pi)
           for j in range(3)] for i in range(3)]
    Ba = [[[((r * Y / 2) * (rh[i] * rh[k] * n[j] + rh[j] * rh[k] * n[i] + kd(j, k) * n[i] + kd(i, k) * n[j])
             + (kd(j, k) * n[i] + kd(i, k) * n[j]) / (2 * s) * (e2 / c2 - e1 / c1) + kd(i, j) * n[k] * e2 / (c2 * s))
            / (4 * mp.pi) for k in range(3)] for j in range(3)] for i in range(3)]
    return U, P, Bt, Ba


def flat(x):
    return [v for row in x for v in (flat(row) if isinstance(row, list) else [row])] if isinstance(x, list) else [x]


def test_stable_forms_equal_literal_formulas():
    mp.mp.dps = 40
    rng = np.random.default_rng(7)
    c1, c2, rho = mp.mpf("11.6"), mp.mpf("6.2"), mp.mpf(1000)
    for _ in range(12):
        rh = [mp.mpf(x) for x in rng.normal(size=3)]
        nr = mp.sqrt(sum(x * x for x in rh))
        rh = [x / nr for x in rh]
        n = [mp.mpf(x) for x in rng.normal(size=3)]
        r = mp.mpf(10 ** rng.uniform(-3, -0.5))
        s = mp.mpc(rng.uniform(10, 300), rng.uniform(-200, 200))
        A, B = literal(r, s, rh, n, c1, c2, rho), stable(r, s, rh, n, c1, c2, rho)
        for qa, qb in zip(A, B):
            fa, fb = flat(qa), flat(qb)
            num = mp.sqrt(sum(abs(x - y) ** 2 for x, y in zip(fa, fb)))
            den = mp.sqrt(sum(abs(x) ** 2 for x in fa))
            assert num / den < mp.mpf(10) ** -30


def test_radial_y_without_psi():
    """Y = psi(z1)/c1^2 - psi(z2)/c2^2 equals ((1 + z1) e1 - (1 + z2) e2) / (s^2 r^2) (c_a^2 z_a^2 =
    s^2 r^2: the -1 of both psi cancel), and psi(z2)/c2^2 = ((1 + z2) e2 - 1) / (s^2 r^2) -- the forms
    the FP32 and compensated radial terms evaluate above the series thresholds."""
    mp.mp.dps = 40
    rng = np.random.default_rng(11)
    psi = lambda z: ((1 + z) * mp.exp(-z) - 1) / (z * z)
    for _ in range(40):
        nu = mp.mpf(rng.uniform(0.2, 0.45))
        c2 = mp.mpf(rng.uniform(2, 20))
        c1 = c2 * mp.sqrt(2 * (1 - nu) / (1 - 2 * nu))
        r = mp.mpf(10 ** rng.uniform(-3, -0.5))
        s = mp.mpc(rng.uniform(10, 400), rng.uniform(-400, 400))
        z1, z2 = r * s / c1, r * s / c2
        e1, e2 = mp.exp(-z1), mp.exp(-z2)
        Y = psi(z1) / c1 ** 2 - psi(z2) / c2 ** 2
        Yc = ((1 + z1) * e1 - (1 + z2) * e2) / (s * s * r * r)
        assert abs(Y - Yc) / abs(Y) < mp.mpf(10) ** -30
        p2 = ((1 + z2) * e2 - 1) / (s * s * r * r)
        assert abs(psi(z2) / c2 ** 2 - p2) / abs(p2) < mp.mpf(10) ** -30


def test_factored_tensor_build():
    """The scatter's per-point tensor build (csrc/sod_collocation.cu, scatter_body; the Galerkin
    regular pairs share it): with the unit coefficients (alpha, beta of G; a, b, d of H) and the
    common factor on the quadrature weight,
        G: u_pq = (alpha rh_p) rh_q + beta d_pq                          times 1/(4 pi rho r)
        H: u_pq = (d rn rh_p + b n_p) rh_q + (a rh_p) n_q + b rn d_pq     times 1/(4 pi r^2)
    equal the literal U and P of the reference; and the B_angular moments kept as two sums,
    sum e1 w and sum e2 w, give the (e2/c2 - e1/c1) moment of the literal form."""
    mp.mp.dps = 40
    rng = np.random.default_rng(19)
    c1, c2, rho = mp.mpf("11.6"), mp.mpf("6.2"), mp.mpf(1000)
    kap = c2 ** 2 / c1 ** 2
    psi = lambda z: ((1 + z) * mp.exp(-z) - 1) / (z * z)
    for _ in range(12):
        rh = [mp.mpf(x) for x in rng.normal(size=3)]
        nr = mp.sqrt(sum(x * x for x in rh))
        rh = [x / nr for x in rh]
        n = [mp.mpf(x) for x in rng.normal(size=3)]
        r = mp.mpf(10 ** rng.uniform(-3, -0.5))
        s = mp.mpc(rng.uniform(10, 300), rng.uniform(-200, 200))
        U, P, _, _ = literal(r, s, rh, n, c1, c2, rho)
        z1, z2 = r * s / c1, r * s / c2
        e1, e2 = mp.exp(-z1), mp.exp(-z2)
        Y = psi(z1) / c1 ** 2 - psi(z2) / c2 ** 2
        rn = sum(rh[k] * n[k] for k in range(3))
        # G: g_coeffs_unit, then the per-row vectors
        Cc = e2 / c2 ** 2
        al, be = 3 * Y + (e1 / c1 ** 2 - Cc), Y * (-1) + Cc
        scG = 1 / (4 * mp.pi * rho) / r
        Uf = [[((al * rh[p]) * rh[q] + (be if p == q else 0)) * scG for q in range(3)] for p in range(3)]
        # H: h_coeffs_unit, then the per-row vectors
        Yc = 6 * c2 ** 2 * Y
        a = Yc + (4 * kap - 1) * e1 - 2 * e2 - (1 - 2 * kap) * z1 * e1
        b = Yc + 2 * kap * e1 - 3 * e2 - z2 * e2
        d = -5 * Yc - 12 * kap * e1 + 12 * e2 - 2 * kap * z1 * e1 + 2 * z2 * e2
        scH = 1 / (4 * mp.pi) / (r * r)
        hdr, hbr = d * rn, b * rn
        Pf = []
        for p in range(3):
            dp, bp = hdr * rh[p] + b * n[p], a * rh[p]
            Pf.append([(dp * rh[q] + (bp * n[q] + hbr if p == q else bp * n[q])) * scH for q in range(3)])
        for A, B in ((U, Uf), (P, Pf)):
            fa, fb = flat(A), flat(B)
            num = mp.sqrt(sum(abs(x - y) ** 2 for x, y in zip(fa, fb)))
            den = mp.sqrt(sum(abs(x) ** 2 for x in fa))
            assert num / den < mp.mpf(10) ** -30
    # the two-sum form of the B_angular (e2/c2 - e1/c1) moment over a face's points
    w = [mp.mpf(x) for x in rng.uniform(0.01, 0.2, size=7)]
    rr = [mp.mpf(10 ** x) for x in rng.uniform(-3, -0.5, size=7)]
    s = mp.mpc(120, 35)
    E1 = [mp.exp(-x * s / c1) for x in rr]
    E2 = [mp.exp(-x * s / c2) for x in rr]
    SB = sum((E2[t] / c2 - E1[t] / c1) * w[t] for t in range(7))
    SE, SC = sum(E1[t] * w[t] for t in range(7)), sum(E2[t] * w[t] for t in range(7))
    assert abs(SB - (SC / c2 - SE / c1)) / abs(SB) < mp.mpf(10) ** -30

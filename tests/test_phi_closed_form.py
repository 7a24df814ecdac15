"""The closed-form composition derivatives of PR76 ln phi used by the FP64
polish (phi_coefficients in pr76_batched.cuh, w64::phi_coeffs), restated in
numpy and checked against central differences of ln phi (CPU only).

    d ln phi_i / d x_j = cs_i s_j + cb_i b_j + ca a_ij
"""

import numpy as np

R = 8.31446261815324
SQ2 = np.sqrt(2.0)


def _model(n, seed):
    rng = np.random.default_rng(seed)
    tc, pc, om = rng.uniform(190, 620, n), rng.uniform(2.5e6, 4.6e6, n), rng.uniform(0.01, 0.35, n)
    k = rng.uniform(0, 0.12, (n, n))
    k = (k + k.T) / 2
    np.fill_diagonal(k, 0.0)
    return tc, pc, om, k


def _state(x, which, T, P, aij, bi):
    s = aij @ x
    a, b = x @ s, x @ bi
    A, B = a * P / (R * T) ** 2, b * P / (R * T)
    r = np.roots([1, -(1 - B), A - 3 * B * B - 2 * B, -(A * B - B * B - B ** 3)])
    r = np.sort(r[np.abs(r.imag) < 1e-12].real)
    r = r[r > B]
    return s, a, b, A, B, (r[0] if which == "l" else r[-1])


def _lnphi(x, which, T, P, aij, bi):
    s, a, b, A, B, Z = _state(x, which, T, P, aij, bi)
    L = np.log((Z + (1 + SQ2) * B) / (Z + (1 - SQ2) * B))
    return bi / b * (Z - 1) - np.log(Z - B) - A / (2 * SQ2 * B) * (2 * s / a - bi / b) * L


def _closed_form(x, which, T, P, aij, bi):
    s, a, b, A, B, Z = _state(x, which, T, P, aij, bi)
    p2 = P / (R * T)
    p1 = p2 / (R * T)
    d1, d2 = Z + (1 + SQ2) * B, Z + (1 - SQ2) * B
    L = np.log(d1 / d2)
    G = A * L / (2 * SQ2 * B)
    fz = (3 * Z - 2 * (1 - B)) * Z + (A - 3 * B * B - 2 * B)
    fa = Z - B
    fb = Z * Z - (6 * B + 2) * Z - A + 2 * B + 3 * B * B
    zs, zb = -2 * fa * p1 / fz, -fb * p2 / fz
    inv = 1 / d1 - 1 / d2
    ls, lb = zs * inv, zb * inv + p2 * ((1 + SQ2) / d1 - (1 - SQ2) / d2)
    gs, gb = (2 * p1 * L + A * ls) / (2 * SQ2 * B), A * lb / (2 * SQ2 * B) - G * p2 / B
    r, q = bi / b, 2 * s / a - bi / b
    cs = r * zs - zs / (Z - B) + 4 * G * s / a ** 2 - q * gs
    cb = -r * (Z - 1) / b + r * zb - (zb - p2) / (Z - B) - G * r / b - q * gb
    return cs[:, None] * s[None, :] + cb[:, None] * bi[None, :] + (-2 * G / a) * aij


def test_closed_form_matches_central_differences():
    for n, seed, T, P in ((3, 1, 300.0, 3e6), (5, 3, 300.0, 3e6), (8, 7, 350.0, 8e6)):
        tc, pc, om, k = _model(n, seed)
        kap = 0.37464 + om * (1.54226 - 0.26992 * om)
        ac = 0.45724 * (R * tc) ** 2 / pc
        bi = 0.07780 * R * tc / pc
        ai = ac * (1 + kap * (1 - np.sqrt(T / tc))) ** 2
        aij = np.sqrt(np.outer(ai, ai)) * (1 - k)
        x = np.random.default_rng(seed).dirichlet(np.ones(n))
        for which in "lv":
            got = _closed_form(x, which, T, P, aij, bi)
            fd = np.zeros((n, n))
            h = 1e-6
            for j in range(n):
                e = np.zeros(n)
                e[j] = h
                fd[:, j] = (_lnphi(x + e, which, T, P, aij, bi) - _lnphi(x - e, which, T, P, aij, bi)) / (2 * h)
            assert np.abs(got - fd).max() <= 1e-7 * np.abs(fd).max(), (n, which)


def _pt_closed_form(x, which, T, P, tc, pc, om, k):
    """d[Z, ln phi]/d[p, T] at fixed x (phase_jacobian_closed in pr76_ad.cuh)."""
    kap = 0.37464 + om * (1.54226 - 0.26992 * om)
    ac = 0.45724 * (R * tc) ** 2 / pc
    bi = 0.07780 * R * tc / pc
    br = 1 + kap * (1 - np.sqrt(T) / np.sqrt(tc))
    ai = ac * br ** 2
    aij = np.sqrt(np.outer(ai, ai)) * (1 - k)
    s, a, b, A, B, Z = _state(x, which, T, P, aij, bi)
    uu = (-kap / (2 * np.sqrt(T) * np.sqrt(tc))) / br
    tt = aij @ (uu * x)
    ap = 2 * np.sum(uu * x * s)
    d1, d2 = Z + (1 + SQ2) * B, Z + (1 - SQ2) * B
    L = np.log(d1 / d2)
    G = A * L / (2 * SQ2 * B)
    fz = (3 * Z - 2 * (1 - B)) * Z + (A - 3 * B * B - 2 * B)
    fa, fb = Z - B, Z * Z - (6 * B + 2) * Z - A + 2 * B + 3 * B * B
    r, q = bi / b, 2 * s / a - bi / b
    out = []
    for dA, dB, dq in ((A / P, B / P, 0 * s), (A * (ap / a - 2 / T), -B / T, 2 * (uu * s + tt) / a - 2 * s * ap / a ** 2)):
        dZ = -(fa * dA + fb * dB) / fz
        dL = (dZ + (1 + SQ2) * dB) / d1 - (dZ + (1 - SQ2) * dB) / d2
        dG = (dA * L + A * dL) / (2 * SQ2 * B) - G * dB / B
        out.append(np.concatenate([[dZ], r * dZ - (dZ - dB) / (Z - B) - dq * G - q * dG]))
    return np.array(out).T, aij, bi


def test_pressure_and_temperature_columns_match_central_differences():
    for n, seed, T, P in ((3, 1, 300.0, 3e6), (6, 5, 330.0, 6e6)):
        tc, pc, om, k = _model(n, seed)
        x = np.random.default_rng(seed + 1).dirichlet(np.ones(n))
        for which in "lv":
            got, _, _ = _pt_closed_form(x, which, T, P, tc, pc, om, k)

            def zl(TT, PP):
                kap = 0.37464 + om * (1.54226 - 0.26992 * om)
                ac = 0.45724 * (R * tc) ** 2 / pc
                bi = 0.07780 * R * tc / pc
                ai = ac * (1 + kap * (1 - np.sqrt(TT / tc))) ** 2
                aij = np.sqrt(np.outer(ai, ai)) * (1 - k)
                Z = _state(x, which, TT, PP, aij, bi)[5]
                return np.concatenate([[Z], _lnphi(x, which, TT, PP, aij, bi)])

            fd_p = (zl(T, P * (1 + 1e-6)) - zl(T, P * (1 - 1e-6))) / (2e-6 * P)
            fd_t = (zl(T * (1 + 1e-6), P) - zl(T * (1 - 1e-6), P)) / (2e-6 * T)
            assert np.abs(got[:, 0] - fd_p).max() <= 1e-6 * np.abs(fd_p).max(), (n, which, "p")
            assert np.abs(got[:, 1] - fd_t).max() <= 1e-6 * np.abs(fd_t).max(), (n, which, "T")

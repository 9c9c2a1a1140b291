"""The FP32-mixed pulse fit's float-float normal-equation solve (csrc/crv_pulsefit.cuh: solve_sym_ff) restated in
NumPy float32 on the CPU: the exact product of two float32 values split into its rounded value and its error (the
device's fmaf; here float64, in which the product of two float32 values is exact), Knuth's exact two-sum, the pairs'
errors carried through the cofactors, the determinant and the adjugate product, the results truncated to float32
and multiplied by the float32 reciprocal of the truncated determinant, as the device does.

On symmetric positive-definite 3x3 systems at the fit's scales (diagonals 1e-2 .. 1e9, correlations up to 0.999999)
the float-float cofactors and determinant are exact to 2^-44 of the sum of their terms' magnitudes (checked against
exact rational arithmetic; FP64 gives 2^-52 of it), and
the float32 solution equals the FP64 solve's (solve_sym64: the same steps in float64): 400 of 400 here, 2,000 of 2,000
in a larger sample; a difference, were there one, would be one float32 rounding."""
from fractions import Fraction

import numpy as np

F = np.float32


def two_prod(a, b):
    p = F(a * b)                                    # round to nearest, as __fmul_rn
    e = F(np.float64(a) * np.float64(b) - np.float64(p))   # exact: the product of two float32 is exact in float64
    return p, e


def two_sum(a, b):
    s = F(a + b)
    bb = F(s - a)
    return s, F(F(a - F(s - bb)) + F(b - bb))


def norm(a, b):
    s = F(a + b)
    return s, F(b - F(s - a))


def mul2m(a, b, c, d):                              # a*b - c*d
    p, q = two_prod(a, b), two_prod(c, d)
    s = two_sum(p[0], F(-q[0]))
    return norm(s[0], F(s[1] + F(p[1] - q[1])))


def fma32(x, y, z):                                 # fmaf: one rounding of x*y + z
    return F(Fraction(float(x)) * Fraction(float(y)) + Fraction(float(z)))


def ffmul(x, y):
    p = two_prod(x, y[0])
    return norm(p[0], fma32(x, y[1], p[1]))


def ffadd(a, b):
    s = two_sum(a[0], b[0])
    return norm(s[0], F(s[1] + F(a[1] + b[1])))


def trunc32(hi, lo):                                # __fadd_rz(hi, lo): the sum rounded toward zero
    x = Fraction(float(hi)) + Fraction(float(lo))
    f = F(float(x))
    if abs(Fraction(float(f))) > abs(x):
        f = np.nextafter(f, F(0))
    return F(f)


def solve_ff(M, b):
    m00, m01, m02, m11, m12, m22 = (F(v) for v in M)
    c00, c01, c02 = mul2m(m11, m22, m12, m12), mul2m(m12, m02, m01, m22), mul2m(m01, m12, m11, m02)
    det = ffadd(ffadd(ffmul(m00, c00), ffmul(m01, c01)), ffmul(m02, c02))
    c11, c12, c22 = mul2m(m00, m22, m02, m02), mul2m(m01, m02, m00, m12), mul2m(m00, m11, m01, m01)
    b0, b1, b2 = (F(v) for v in b)
    y = [ffadd(ffadd(ffmul(b0, c00), ffmul(b1, c01)), ffmul(b2, c02)),
         ffadd(ffadd(ffmul(b0, c01), ffmul(b1, c11)), ffmul(b2, c12)),
         ffadd(ffadd(ffmul(b0, c02), ffmul(b1, c12)), ffmul(b2, c22))]
    r = F(F(1) / trunc32(*det))
    return np.array([F(trunc32(*v) * r) for v in y]), (c00, c01, c02, c11, c12, c22, det)


def solve_64(M, b):
    m00, m01, m02, m11, m12, m22 = (np.float64(F(v)) for v in M)
    c00, c01, c02 = m11 * m22 - m12 * m12, m12 * m02 - m01 * m22, m01 * m12 - m11 * m02
    det = m00 * c00 + m01 * c01 + m02 * c02
    c11, c12, c22 = m00 * m22 - m02 * m02, m01 * m02 - m00 * m12, m00 * m11 - m01 * m01
    b0, b1, b2 = (np.float64(F(v)) for v in b)
    y = [c00 * b0 + c01 * b1 + c02 * b2, c01 * b0 + c11 * b1 + c12 * b2, c02 * b0 + c12 * b1 + c22 * b2]

    def t32(x):                                     # d2f_trunc: float64 -> float32 toward zero
        f = F(x)
        return np.nextafter(f, F(0)) if abs(np.float64(f)) > abs(x) else f
    r = F(F(1) / t32(det))
    return np.array([F(t32(v) * r) for v in y])


def _systems(n, rng):
    out = []
    for _ in range(n):
        s = 10.0 ** rng.uniform(-1, 4.5, 3)                 # column scales: diagonals 1e-2 .. 1e9
        c = rng.uniform(-1, 1, (3, 3))
        c = c @ c.T + np.eye(3) * 10.0 ** rng.uniform(-6, 0)
        d = np.sqrt(np.diag(c))
        c = c / np.outer(d, d)                              # correlations, some very close to 1
        M = c * np.outer(s, s)
        b = rng.normal(size=3) * s * 10.0 ** rng.uniform(-3, 1)
        out.append(([M[0, 0], M[0, 1], M[0, 2], M[1, 1], M[1, 2], M[2, 2]], b))
    return out


def test_float_float_cofactors_carry_46_bits_and_match_the_fp64_solve():
    rng = np.random.default_rng(17)
    same = 0
    systems = _systems(400, rng)
    for M, b in systems:
        x, parts = solve_ff(M, b)
        m = [Fraction(float(F(v))) for v in M]
        # each quantity with the sum of the magnitudes of its terms: a float-float result is exact to ~2^-46 of it
        pairs = {"c00": (m[3] * m[5], m[4] * m[4]), "c01": (m[4] * m[2], m[1] * m[5]),
                 "c02": (m[1] * m[4], m[3] * m[2]), "c11": (m[0] * m[5], m[2] * m[2]),
                 "c12": (m[1] * m[2], m[0] * m[4]), "c22": (m[0] * m[3], m[1] * m[1])}
        exact = {k: (a - c, abs(a) + abs(c)) for k, (a, c) in pairs.items()}
        terms = [m[0] * exact["c00"][0], m[1] * exact["c01"][0], m[2] * exact["c02"][0]]
        exact["det"] = (sum(terms), sum(abs(t) for t in terms) + abs(m[0]) * exact["c00"][1] +
                        abs(m[1]) * exact["c01"][1] + abs(m[2]) * exact["c02"][1])
        for (k, (e, mag)), (hi, lo) in zip(exact.items(), parts):
            err = abs(Fraction(float(hi)) + Fraction(float(lo)) - e)
            assert err <= mag * Fraction(1, 2 ** 44), k
        y = solve_64(M, b)
        if np.array_equal(x, y):
            same += 1
        else:                                               # one float32 rounding apart at most
            ulp = np.spacing(np.abs(y).astype(F)).astype(np.float64)
            assert np.all(np.abs(x.astype(np.float64) - y) <= 2 * ulp + 1e-30)
    assert same >= 0.99 * len(systems)

"""The float-pair error model of the speculative kernels, restated in numpy float32.

The kernels decide the reference's binary64 choice and clock from float-pair
propensities and a float32 running sum (rebop_gb300/csrc/ssa_spec_body.cuh:
df_mul_fu, rs_add, rs_total).  These tests replay those operations with IEEE
float32 arithmetic on random networks and check the bounds the kernels rely
on against exact rational arithmetic: the running sums' high parts within
(r + M + 2) 2^-24 of the exact running sums, and the total within
G = (M + R + 2 + (R (R + 1) / 2 + R (M + 2)) / 16) 2^-44.
"""

from fractions import Fraction

import numpy as np

f32 = np.float32


def fma32(a, b, c):
    # a*b is exact in binary64 for float32 operands; the sum is rounded once
    # to binary64 and then to float32 (double rounding can move the last bit,
    # far below the bounds checked here)
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def df_from_double(v):
    h = np.float32(v)
    if abs(np.float64(h)) > abs(v):  # truncate toward zero, as __double2float_rz
        h = np.nextafter(h, f32(0))
    return h, f32(v - np.float64(h))


def df_mul_fu(a, f):
    p = f32(a[0] * f)
    return p, fma32(a[1], f, fma32(a[0], f, -p))


def rs_add(s, e, b):
    s2 = f32(s + b[0])
    bb = f32(s2 - s)
    err = f32(f32(s - f32(s2 - bb)) + f32(b[0] - bb))
    return s2, f32(e + f32(err + b[1]))


def fast2sum(a, b):
    s = f32(a + b)
    return s, f32(b - f32(s - a))


def test_running_sums_and_total_within_their_bounds():
    rng = np.random.default_rng(2026)
    for _ in range(1500):
        R = int(rng.integers(1, 33))
        M = int(rng.integers(1, 4))
        rates = np.exp(rng.uniform(np.log(1e-6), np.log(1e6), R))
        orders = rng.integers(0, M + 1, R)
        counts = rng.integers(0, 1 << int(rng.integers(1, 23)), R)
        s, e = f32(0), f32(0)
        exact_run = Fraction(0)
        highs, exacts = [], []
        for r in range(R):
            acc = df_from_double(rates[r])
            ex = Fraction(float(rates[r]))
            for j in range(int(orders[r])):
                x = max(int(counts[r]) - j, 0)
                acc = df_mul_fu(acc, f32(x))
                ex *= x
            s, e = rs_add(s, e, acc)
            exact_run += ex
            highs.append(Fraction(float(s)))
            exacts.append(exact_run)
        tot = fast2sum(s, e)
        total = exacts[-1]
        for r, (h, x) in enumerate(zip(highs, exacts), 1):
            assert abs(h - x) <= Fraction(r + M + 2, 1 << 24) * x + Fraction(0), (R, M, r)
        if total > 0:
            G = (M + R + 2 + (R * (R + 1) / 2 + R * (M + 2)) / 16) * 2.0**-44
            got = Fraction(float(tot[0])) + Fraction(float(tot[1]))
            assert abs(got - total) <= Fraction(G) * total, (R, M)


def f32_rz(v):
    h = np.float32(v)
    if abs(np.float64(h)) > abs(v):
        h = np.nextafter(h, f32(0))
    return h


def test_float32_wedge_test_decides_as_binary64(O):
    # The ziggurat's wedge test f[i+1] + (f[i] - f[i+1]) U < exp(-x), decided
    # in float32 outside a 2^-17 band (wedge_df in ssa_spec_body.cuh), must
    # agree with the binary64 test of the oracle's sampler whenever it
    # decides.  x = (2k + 1) 2^-53 X[i] and U = mu 2^-53 as drawn; exp here is
    # numpy's float32 exp, within the 2 ulp the band allows for expf.
    X, F = O.zig_tables()
    rng = np.random.default_rng(11)
    decided = band = 0
    for i in range(1, 256):
        zd = F[i + 1] - F[i]
        assert zd > 0
        for _ in range(400):
            k = int(rng.integers(0, 1 << 52))
            mu = int(rng.integers(0, 1 << 53))
            x = ((2 * k + 1) * 2.0**-53) * X[i]
            U = mu * 2.0**-53
            exact = F[i + 1] + (F[i] - F[i + 1]) * U < np.exp(-x)
            u = f32(f32((mu >> 30) & 0x7FFFFF) * f32(2.0**-23))
            wf = fma32(-f32_rz(zd), u, f32_rz(F[i + 1]))
            ef = np.exp(-f32(x), dtype=np.float32)
            if wf < f32(ef * f32(1 - 2.0**-17)):
                decided += 1
                assert exact, (i, k, mu)
            elif wf > f32(ef * f32(1 + 2.0**-17)):
                decided += 1
                assert not exact, (i, k, mu)
            else:
                band += 1
    assert decided > 100 * band

"""Accuracy of the float-float algorithms the refresh kernels use, restated
step for step in numpy float32 arithmetic (round-to-nearest, exact FMA) and
checked against mpmath:

  * exp (qmc_ff.cuh): Tang's table method, ln2/32 reduction, 32-entry table;
  * erfc on [0, 6] (qmc_heg_kernels.cuh): Chebyshev series by Clenshaw, FP32
    tail from k = 24;
  * sine and cosine (qmc_heg_kernels.cuh): three-part pi/2 reduction, split
    Taylor series.

The device code itself is checked by the GPU parity tests (E_L and log|psi|
against the FP64 oracle); these tests pin the error bounds stated beside
each algorithm.
"""
import os
import sys

import numpy as np
import pytest

mp = pytest.importorskip("mpmath")

f32 = np.float32


def fma(a, b, c):
    return f32(np.float64(a) * np.float64(b) + np.float64(c))   # float32 products are exact in float64


def two_sum(a, b):
    s = f32(a + b)
    bb = f32(s - a)
    return s, f32(f32(a - f32(s - bb)) + f32(b - bb))


def fast_two_sum(a, b):
    s = f32(a + b)
    return s, f32(b - f32(s - a))


def two_prod(a, b):
    p = f32(a * b)
    return p, fma(a, b, -p)


def add(a, b):
    s, e = two_sum(a[0], b[0])
    return fast_two_sum(s, f32(e + f32(a[1] + b[1])))


def neg(a):
    return f32(-a[0]), f32(-a[1])


def mul(a, b):
    p, e = two_prod(a[0], b[0])
    e = fma(a[0], b[1], e)
    e = fma(a[1], b[0], e)
    return fast_two_sum(p, e)


def of(x):
    x = mp.mpf(x)
    hi = f32(float(x))
    return hi, f32(float(x - mp.mpf(float(hi))))


def value(a):
    return mp.mpf(float(a[0])) + mp.mpf(float(a[1]))


def ff_exp(a):
    tab = [of(mp.mpf(2) ** (mp.mpf(j) / 32)) for j in range(32)]
    ln2_32 = of(mp.log(2) / 32)
    n = f32(np.rint(f32(a[0] * f32(46.166241308446828))))
    p, pe = two_prod(ln2_32[0], n)
    t = fast_two_sum(p, fma(ln2_32[1], n, pe))
    r = add(a, neg(t))
    q, qe = two_prod(r[0], r[0])
    h = (f32(q * f32(0.5)), f32(fma(f32(2 * r[0]), r[1], qe) * f32(0.5)))
    poly = fma(r[0], fma(r[0], f32(1 / 60), f32(1 / 12)), f32(1 / 3))
    s = add(h, (f32(f32(h[0] * r[0]) * poly), f32(0)))
    s = add(r, s)
    s = add((f32(1), f32(0)), s)
    m = mul(s, tab[int(n) & 31])
    sc = f32(2.0 ** (int(n) >> 5))
    return f32(m[0] * sc), f32(m[1] * sc)


_ERFC = []


def erfc_coefficients():
    if not _ERFC:
        sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "rust_qmc_gb300", "csrc"))
        import gen_erfc_table as G
        _ERFC.extend(G.coefficients())
    return _ERFC


def ff_erfc(x):
    c = erfc_coefficients()
    if not x[0] < 6:
        return f32(0), f32(0)
    t = add(mul(x, of(mp.mpf(1) / 3)), (f32(-1), f32(0)))
    b1 = b2 = f32(0)
    for k in range(42, 23, -1):
        b0 = fma(f32(2 * t[0]), b1, f32(f32(float(c[k])) - b2))
        b2, b1 = b1, b0
    B1, B2 = (b1, f32(0)), (b2, f32(0))
    t2 = (f32(2 * t[0]), f32(2 * t[1]))
    for k in range(23, 0, -1):
        B0 = add(add(mul(t2, B1), of(c[k])), neg(B2))
        B2, B1 = B1, B0
    c0 = of(c[0])
    return add(add((f32(0.5 * c0[0]), f32(0.5 * c0[1])), mul(t, B1)), neg(B2))


def ff_sincos(x):
    n = f32(np.rint(f32(x[0] * f32(0.63661975))))
    p, q = two_prod(f32(1.5707964), n), two_prod(f32(-4.371139e-08), n)
    r = add((f32(x[0] - p[0]), f32(0)), (x[1], f32(0)))
    r = add(r, (f32(-p[1]), f32(0)))
    r = add(r, neg(q))
    r = add(r, (f32(-f32(f32(-1.7151245e-15) * n)), f32(0)))
    r2 = mul(r, r)
    h2 = r2[0]
    qs = f32(h2 * fma(h2, fma(h2, f32(1.6059044e-10), f32(-2.5052108e-08)), f32(2.7557319e-06)))
    cs = add(of(mp.mpf(-1) / 5040), (qs, f32(0)))
    cs = add(mul(cs, r2), of(mp.mpf(1) / 120))
    cs = add(mul(cs, r2), of(mp.mpf(-1) / 6))
    sn = add(r, mul(mul(cs, r2), r))
    qc = fma(h2, fma(h2, fma(h2, f32(4.7794773e-14), f32(-1.1470746e-11)), f32(2.0876757e-09)), f32(-2.7557319e-07))
    cc = add(of(mp.mpf(1) / 40320), (f32(qc * h2), f32(0)))
    cc = add(mul(cc, r2), of(mp.mpf(-1) / 720))
    cc = add(mul(cc, r2), of(mp.mpf(1) / 24))
    cc = add(mul(cc, r2), of(mp.mpf(-1) / 2))
    cn = add((f32(1), f32(0)), mul(cc, r2))
    return [(sn, cn), (cn, neg(sn)), (neg(sn), neg(cn)), (neg(cn), sn)][int(n) & 3]


def test_exp_relative_error():
    mp.mp.dps = 30
    rng = np.random.default_rng(1)
    worst = 0
    for x in np.concatenate([rng.uniform(-60, 0, 400), rng.uniform(-1, 5, 200)]):
        a = of(x)
        worst = max(worst, abs(value(ff_exp(a)) / mp.exp(value(a)) - 1))
    assert worst < 5e-13, worst


def test_erfc_absolute_error():
    mp.mp.dps = 30
    worst = 0
    for x in np.concatenate([np.linspace(0, 6, 241), np.random.default_rng(2).uniform(0, 6, 200)]):
        a = of(x)
        worst = max(worst, abs(value(ff_erfc(a)) - mp.erfc(value(a))))
    assert worst < 2e-14, worst


def test_sincos_absolute_error():
    mp.mp.dps = 30
    rng = np.random.default_rng(3)
    worst = 0
    for x in np.concatenate([rng.uniform(-60, 60, 600), np.linspace(-0.8, 0.8, 81)]):
        a = of(x)
        s, c = ff_sincos(a)
        worst = max(worst, abs(value(s) - mp.sin(value(a))), abs(value(c) - mp.cos(value(a))))
    assert worst < 1e-13, worst

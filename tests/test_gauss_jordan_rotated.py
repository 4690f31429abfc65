"""The warp Gauss-Jordan inversion of the benzene and electron-gas refresh
kernels (kw_measure_walker in qmc_warp_kernels.cuh, khw_measure_walker in
qmc_heg_kernels.cuh), restated step for step in numpy: lane j of a warp holds
column j, the pivot loop is rolled with the rows rotated one register per
step (row k in register 0 at step k, the rows not yet pivoted first), pivots
are chosen on the leading parts, and the row interchanges are undone at the
end as a gather of columns src(j).

These tests pin the bookkeeping (rotation, pivot offsets, the src
permutation, the determinant's sign) against numpy's inverse and determinant
for full and padded sectors; the device arithmetic itself is checked by the
GPU parity tests.
"""
import numpy as np
import pytest

LANES = 32


def warp_gauss_jordan(D, nm):
    """Invert the ns x ns matrix D as the kernels do, with nm register rows
    (nm >= ns; rows and lanes beyond ns hold the identity).  Returns the
    inverse, log|det| and the sign of det (real input) or 0 (complex)."""
    ns = D.shape[0]
    cplx = np.iscomplexobj(D)
    R = np.zeros((nm, LANES), dtype=D.dtype)
    for i in range(nm):
        for lane in range(LANES):
            R[i, lane] = D[i, lane] if (i < ns and lane < ns) else (1 if i == lane else 0)
    src = np.arange(LANES)
    logdet, sign = 0.0, 1
    lead = (lambda z: np.float32(z.real) ** 2 + np.float32(z.imag) ** 2) if cplx else (lambda x: abs(np.float32(x)))
    for k in range(ns):
        # pivot over the rows not yet pivoted: registers 0 .. ns-1-k
        p, best = 0, lead(R[0, k])
        for r in range(1, nm):
            m = lead(R[r, k])
            if r < ns - k and m > best:
                best, p = m, r
        R[[0, p]] = R[[p, 0]]
        if p != 0:
            sign = -sign
        pk = k + p
        src = np.where(src == k, pk, np.where(src == pk, k, src))
        piv = R[0, k]
        assert piv != 0
        if not cplx and piv < 0:
            sign = -sign
        logdet += np.log(abs(piv))
        ip = 1 / piv
        t = R[0] * ip
        t[k] = 1 + ip
        R[0] = t
        R[0, k] = ip
        for i in range(1, nm):
            if i < ns:
                R[i] = R[i] - R[i, k] * t
        # rotate registers 0..ns-1 by one
        R[:ns] = np.roll(R[:ns], -1, axis=0)
    R = R[:, src]                      # lane j gathers column src(j)
    return R[:ns, :ns], logdet, (0 if cplx else sign)


@pytest.mark.parametrize("nm,ns", [(21, 21), (27, 27), (6, 4), (5, 1)])
def test_real_inverse_logdet_sign(nm, ns):
    rng = np.random.default_rng(nm * 100 + ns)
    for _ in range(3):
        D = rng.normal(size=(ns, ns))
        inv, logdet, sign = warp_gauss_jordan(D, nm)
        s, ld = np.linalg.slogdet(D)
        assert np.allclose(inv, np.linalg.inv(D), rtol=1e-9, atol=1e-10)
        assert logdet == pytest.approx(ld, rel=1e-12, abs=1e-12)
        assert sign == int(s)


@pytest.mark.parametrize("nm,ns", [(27, 27), (7, 5)])
def test_complex_inverse_logdet(nm, ns):
    rng = np.random.default_rng(nm + ns)
    D = rng.normal(size=(ns, ns)) + 1j * rng.normal(size=(ns, ns))
    inv, logdet, _ = warp_gauss_jordan(D, nm)
    assert np.allclose(inv, np.linalg.inv(D), rtol=1e-9, atol=1e-10)
    assert logdet == pytest.approx(np.linalg.slogdet(D)[1], rel=1e-12, abs=1e-12)


def test_pivoting_handles_zero_leading_entries():
    # a permutation-like matrix: without row interchanges the first pivot is 0
    ns = 8
    rng = np.random.default_rng(3)
    perm = rng.permutation(ns)
    D = np.eye(ns)[perm] * rng.uniform(1, 2, size=ns)
    inv, logdet, sign = warp_gauss_jordan(D, ns)
    s, ld = np.linalg.slogdet(D)
    assert np.allclose(inv, np.linalg.inv(D))
    assert sign == int(s) and logdet == pytest.approx(ld)


def test_rotation_returns_rows_to_their_order():
    # the identity needs no interchanges: after ns rotations register k holds row k
    ns = 11
    inv, logdet, sign = warp_gauss_jordan(np.diag(np.arange(1.0, ns + 1)), ns)
    assert np.allclose(inv, np.diag(1 / np.arange(1.0, ns + 1)))
    assert sign == 1

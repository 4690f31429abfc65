"""Twist-averaged boundary conditions for the electron gas (host side):
Monkhorst-Pack grids and twisted plane-wave sets restate
src/systems/heg.rs:176-232; the averages restate examples/heg_vmc.rs:178-186."""
import math

import numpy as np
import pytest

import rust_qmc_gb300 as Q
from rust_qmc_gb300.twist import average_twists


def test_monkhorst_pack_grid():
    assert np.array_equal(Q.monkhorst_pack_grid(1), [[0.0, 0.0, 0.0]])
    g2 = Q.monkhorst_pack_grid(2)
    assert g2.shape == (8, 3)
    assert np.array_equal(g2[0], [-0.25, -0.25, -0.25]) and np.array_equal(g2[1], [-0.25, -0.25, 0.25])
    assert np.array_equal(g2[7], [0.25, 0.25, 0.25])
    g3 = Q.monkhorst_pack_grid(3)
    assert g3.shape == (27, 3)
    np.testing.assert_allclose(sorted(set(g3[:, 0])), [-1.0 / 3.0, 0.0, 1.0 / 3.0], atol=1e-15)
    np.testing.assert_allclose(g3.mean(0), 0.0, atol=1e-15)


def brute_force_k(n, L, twist):
    m = int(math.ceil(n ** (1.0 / 3.0) * 2.0)) + 2
    dk = 2.0 * math.pi / L
    r = np.arange(-m, m + 1, dtype=np.float64)
    g = np.stack(np.meshgrid(r, r, r, indexing="ij"), -1).reshape(-1, 3)
    k = g * dk + np.asarray(twist) * dk
    k2 = k[:, 0] * k[:, 0] + k[:, 1] * k[:, 1] + k[:, 2] * k[:, 2]
    return k[np.argsort(k2, kind="stable")[:n]]


def test_twisted_k_vectors_are_the_lowest_shifted_waves():
    for twist in [(0.25, -0.1, 0.4), (0.5, 0.5, 0.5), (-1.0 / 3.0, 0.0, 1.0 / 3.0)]:
        for n, L in [(27, 12.0), (7, 5.3), (33, 19.5)]:
            assert np.array_equal(Q.heg_k_vectors(n, L, twist), brute_force_k(n, L, twist))
    assert np.array_equal(Q.heg_k_vectors(27, 12.0, (0.0, 0.0, 0.0)), Q.heg_k_vectors(27, 12.0))


def test_electron_gas_twist_shifts_both_spin_sets():
    g0 = Q.electron_gas()
    th = np.array([0.25, -0.25, 0.25])
    g1 = Q.electron_gas(twist=th)
    dk = 2.0 * math.pi / g1.box_L
    k0, k1 = np.asarray(g0.mo_coef).reshape(-1, 3), np.asarray(g1.mo_coef).reshape(-1, 3)
    assert k1.shape == k0.shape
    frac = k1 / dk - th                       # integer lattice vectors
    np.testing.assert_allclose(frac, np.round(frac), atol=1e-12)
    assert np.array_equal(g1.occ, g0.occ) and g1.box_L == g0.box_L


def test_average_twists_matches_reference_formula():
    e, s = [-1.0, -1.2, -0.9, -1.1], [0.01, 0.02, 0.015, 0.01]
    avg, err, err_mean = average_twists(e, s)
    assert avg == sum(e) / 4
    assert err == math.sqrt(sum(x * x for x in s) / 4)
    assert err_mean == math.sqrt(sum(x * x for x in s)) / 4


def test_hartree_fock_energy_ranges():
    """The reference's own check (src/systems/heg.rs:1027-1038): E_HF/N in
    (0.5, 1.0) Ha at r_s = 1 and in (-0.1, 0) at r_s = 4; the closed form
    1.105/r_s^2 - 0.458/r_s of its docstring."""
    from rust_qmc_gb300.twist import hartree_fock_energy
    assert 0.5 < hartree_fock_energy(1.0) < 1.0
    assert -0.1 < hartree_fock_energy(4.0) < 0.0
    for rs in (1.0, 2.0, 4.0, 10.0):
        assert abs(hartree_fock_energy(rs) - (1.105 / rs ** 2 - 0.458 / rs)) < 2e-3 / rs


def test_correlation_fit_is_continuous_at_rs_one():
    """The two branches of the Perdew-Zunger fit meet at r_s = 1 (heg.rs:834-849)."""
    from rust_qmc_gb300.twist import correlation_energy
    assert abs(correlation_energy(1.0) - correlation_energy(1.0 - 1e-9)) < 1e-4
    assert correlation_energy(4.0) == pytest.approx(-0.1423 / (1 + 1.0529 * 2 + 0.3334 * 4))
    assert correlation_energy(0.5) < correlation_energy(4.0) < 0

"""CPU checks that pin the oracle to the reference.

The reference (a Rust crate) cannot be built here, so the oracle is pinned by
the reference's own golden scalars, its finite-difference self-consistency
tests, its range checks, and the published Philox known-answer vectors.
"""
import math

import numpy as np
import pytest

import rust_qmc_gb300 as Q
from tests.helpers import fd_grad_lap, random_configs


# Philox4x32-10 known-answer vectors (Random123 distribution, kat_vectors).
KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


@pytest.mark.parametrize("ctr,key,want", KAT)
def test_philox_known_answers(oracle, ctr, key, want):
    assert oracle.philox(ctr, key) == want
    assert Q.philox4x32(ctr, key) == want


def test_descriptor_layout_matches_abi(oracle):
    import ctypes
    assert oracle.lib().orc_desc_size() == ctypes.sizeof(Q._lib.SystemDesc)


def test_jastrow1_golden(oracle):
    # src/lib.rs:31-56: Jastrow1(F=1) at r1=0, r2=(1,0,0)
    spec = Q.h2_mo(F=1.0)
    r = np.array([[0.0, 0, 0], [1.0, 0, 0]])
    J, g, _ = oracle.jastrow(spec, r)
    assert abs(J - 0.7788007831) < 1e-8
    assert abs(g[0, 0] - (-0.09735009789)) < 1e-6 and abs(g[1, 0] - 0.09735009789) < 1e-6
    assert np.all(np.abs(g[:, 1:]) < 1e-12)


def test_jastrow1_symmetry_translation(oracle):
    # src/lib.rs:69-85
    spec = Q.h2_mo(F=1.0)
    r = np.array([[0.5, 0.5, 0.5], [-0.5, -0.5, -0.5]])
    J1, g, _ = oracle.jastrow(spec, r)
    J2, _, _ = oracle.jastrow(spec, r[::-1].copy())
    assert abs(J1 - J2) < 1e-12
    assert np.linalg.norm(g[0] + g[1]) < 1e-12


@pytest.mark.parametrize("builder", ["h2", "li_fixed", "ch4_gto", "ch4_min"])
def test_oracle_analytic_vs_fd(oracle, builder):
    """Analytic gradient/Laplacian vs central differences (src/lib.rs:88-267,
    src/systems/methane.rs:1310-1337), on seeded configurations."""
    spec = {"h2": lambda: Q.h2_mo(), "li_fixed": lambda: Q.lithium_atom(reference_quirks=False),
            "ch4_gto": lambda: Q.methane_gto(), "ch4_min": lambda: Q.methane_minimal()}[builder]()
    cfgs = random_configs(spec, 3, seed=11)
    ev = oracle.evaluate(spec, cfgs)
    for w in range(3):
        g, l = fd_grad_lap(oracle, spec, cfgs[w], h=2e-5)
        np.testing.assert_allclose(ev["grad"][w], g, rtol=1e-5, atol=1e-5 * (1 + np.abs(g).max()))
        np.testing.assert_allclose(ev["lap"][w], l, rtol=1e-3, atol=1e-3 * (1 + np.abs(l).max()))


def test_lithium_quirks_reproduce_reference_formulas(oracle):
    """With the Jastrow2 quirks on, grad J2 / J2 carries F/(2(1+r/F)^2 r) per
    pair (src/correlation/jastrow.rs:102) and lap J2 / J2 the per-pair sum
    without cross terms (:110-125)."""
    spec = Q.lithium_atom(F=2.0, reference_quirks=True)
    r = random_configs(spec, 1, seed=5)[0]
    J, g, l = oracle.jastrow(spec, r)
    F = 2.0
    gw = np.zeros((3, 3))
    lw = np.zeros(3)
    u = 0.0
    for i in range(3):
        for j in range(i + 1, 3):
            rij = r[i] - r[j]
            d = np.linalg.norm(rij)
            f = 1 + d / F
            u += -F / (2 * f)
            gi = F / (2 * f * f * d) * rij
            gw[i] += gi
            gw[j] -= gi
            comp = (2 * f * f) ** -2 + 1 / (d * f ** 3)
            lw[i] += comp
            lw[j] += comp
    assert abs(J - math.exp(u)) < 1e-14
    np.testing.assert_allclose(g, J * gw, rtol=1e-12)
    np.testing.assert_allclose(l, J * lw, rtol=1e-12)


@pytest.mark.parametrize("builder", ["ch4_gto", "ch4_min", "c6h6"])
def test_log_derivatives_vs_fd(oracle, builder):
    """O_p = d ln|psi| / dp vs central differences (src/systems/methane.rs:
    1340-1373, benzene.rs:976-1006), all 8 Jastrow parameters and the
    MO-rotation angles."""
    spec = {"ch4_gto": lambda: Q.methane_gto(2.0, 3.0), "ch4_min": Q.methane_minimal,
            "c6h6": Q.benzene_minimal}[builder]()
    if builder == "ch4_min":
        spec = spec.with_params(np.concatenate([spec.jas, [0.1, -0.2, 0.05, 0.3]]))
    r = random_configs(spec, 2, seed=3)
    O = oracle.log_derivatives(spec, r)
    p0 = spec.params()
    h = 1e-5
    for k in range(spec.n_params):
        pp, pm = p0.copy(), p0.copy()
        pp[k] += h
        pm[k] -= h
        lp = oracle.evaluate(spec.with_params(pp), r)["logabs"]
        lm = oracle.evaluate(spec.with_params(pm), r)["logabs"]
        fd = (lp - lm) / (2 * h)
        np.testing.assert_allclose(O[:, k], fd, rtol=1e-6, atol=1e-7)


@pytest.mark.parametrize("builder", ["ch4_gto", "c6h6"])
def test_reference_four_parameter_derivatives(oracle, builder):
    """The four log-derivatives d_ln_j_d_{bee,ben,a_anti,a_para} of MethaneGTO
    and BenzeneGTO's OptimizableWfn (src/correlation/jastrow.rs:326-391,
    src/systems/benzene.rs:726-756) are sums of the generalised derivatives,
    checked by FD with b_anti=b_para and B0=B1 tied as in the reference."""
    spec = Q.methane_gto(2.0, 3.0) if builder == "ch4_gto" else Q.benzene_minimal()
    r = random_configs(spec, 1, seed=9)
    O = oracle.log_derivatives(spec, r)[0]
    ref4 = [O[0] + O[1], O[4] + O[5], O[2], O[3]]
    p = Q.reference_params_from_general(spec.params())
    h = 1e-5
    for k in range(4):
        pp, pm = list(p), list(p)
        pp[k] += h
        pm[k] -= h
        sp = spec.with_params(Q.jastrow3_params(pp[0], pp[1], pp[2], pp[3]))
        sm = spec.with_params(Q.jastrow3_params(pm[0], pm[1], pm[2], pm[3]))
        fd = (oracle.evaluate(sp, r)["logabs"][0] - oracle.evaluate(sm, r)["logabs"][0]) / (2 * h)
        assert abs(ref4[k] - fd) <= 1e-6 * max(1.0, abs(fd))


@pytest.mark.parametrize("builder", ["h2", "ch4_gto", "ch4_min", "c6h6"])
def test_nuclear_gradient_vs_fd(oracle, builder):
    """Analytic d ln|psi| / dR_I (src/systems/methane.rs:1007-1101) vs the FD
    form of src/systems/hydrogen.rs:260-290.  For benzene the oracle's form
    is an extension: the reference's BenzeneGTO keeps the trait's
    unimplemented wfn_nuclear_gradient (src/sampling/traits.rs:50-55) and
    implements only the Hellmann-Feynman force (benzene.rs:828-858)."""
    spec = {"h2": lambda: Q.h2_mo(), "ch4_gto": lambda: Q.methane_gto(), "ch4_min": lambda: Q.methane_minimal(),
            "c6h6": lambda: Q.benzene_minimal()}[builder]()
    r = random_configs(spec, 2, seed=21)
    _, Om = oracle.forces(spec, r)
    fd = oracle.nuclear_gradient_fd(spec, r, h=1e-5)
    np.testing.assert_allclose(Om, fd, rtol=1e-5, atol=1e-6)


def test_hf_force_sum_rule(oracle):
    """HF forces (src/systems/methane.rs:1241-1272): the nuclear-nuclear part
    is antisymmetric, so sum_I F_I equals the total electron-nucleus pull."""
    spec = Q.methane_gto()
    r = random_configs(spec, 1, seed=4)
    F, _ = oracle.forces(spec, r)
    tot = np.zeros(3)
    for I in range(spec.n_nuc):
        for i in range(spec.n_elec):
            d = r[0, i] - spec.nuc_pos[I]
            tot += spec.nuc_charge[I] * d / np.linalg.norm(d) ** 3
    np.testing.assert_allclose(F[0].sum(axis=0), tot, rtol=1e-12, atol=1e-12)


def test_methane_ranges():
    """src/systems/methane.rs:1284-1307: C-H 2.05 bohr, tetrahedral, V_nn in (10, 20)."""
    spec = Q.methane_gto()
    R = spec.nuc_pos
    for h in range(1, 5):
        assert abs(np.linalg.norm(R[h] - R[0]) - 2.05) < 1e-12
    hh = [np.linalg.norm(R[i] - R[j]) for i in range(1, 5) for j in range(i + 1, 5)]
    assert max(hh) - min(hh) < 1e-12
    assert 10.0 < spec.v_nn() < 20.0


def test_benzene_ranges():
    """The reference's benzene checks (src/systems/benzene.rs:871-913,926-932)
    on the benzene workload: carbons on a ring of radius C-C = 2.64 bohr,
    C-C-C angles 120 degrees, a planar molecule, C-H 2.05 bohr (the
    workload's bond; the reference builds 2.042), V_nn in (180, 230) Ha,
    and 36 AOs for 21 doubly occupied MOs (the reference: 66 AOs, 6-31G)."""
    spec = Q.benzene_minimal()
    R, Z = spec.nuc_pos, spec.nuc_charge
    C = R[Z == 6]
    H = R[Z == 1]
    assert len(C) == 6 and len(H) == 6 and spec.n_elec == 42
    cc = 2.64
    for i in range(6):
        assert abs(np.linalg.norm(C[i]) - cc) < 1e-10
        assert abs(np.linalg.norm(C[i] - C[(i + 1) % 6]) - cc) < 0.01
        v1 = C[(i + 5) % 6] - C[i]
        v2 = C[(i + 1) % 6] - C[i]
        ang = math.degrees(math.acos(v1 @ v2 / np.linalg.norm(v1) / np.linalg.norm(v2)))
        assert abs(ang - 120.0) < 0.1
    assert np.all(np.abs(R[:, 2]) < 1e-10)
    for i in range(6):
        assert abs(min(np.linalg.norm(H[i] - c) for c in C) - 2.05) < 0.01
    assert 180.0 < spec.v_nn() < 230.0
    occ = np.asarray(spec.occ)
    assert len(spec.ao_nuc) == 36 and sorted(set(occ.tolist())) == list(range(21))
    assert np.sum(np.asarray(spec.spins) > 0) == 21


def test_synthetic_mo_orthonormal():
    spec = Q.methane_minimal()
    M = spec.mo_coef
    np.testing.assert_allclose(M @ M.T, np.eye(9), atol=1e-13)
    assert spec.n_params == 12


def test_oracle_init_matches_layout(oracle):
    """Initial positions: electron e at N(R_init(e), sigma) from the tag-3
    Philox stream (src/systems/methane.rs:1105-1120 placement)."""
    spec = Q.methane_gto()
    pos = oracle.init_positions(spec, 4, seed=123)
    x = Q.philox4x32((2, 0, 7, 3), (123, 0))
    u1, u2 = (x[0] + 0.5) / 2 ** 32, (x[1] + 0.5) / 2 ** 32
    n0 = math.sqrt(-2 * math.log(u1)) * math.cos(2 * math.pi * u2)
    assert abs(pos[2, 7, 0] - (spec.nuc_pos[1, 0] + 0.5 * n0)) < 1e-12


def test_oracle_sweeps_deterministic(oracle):
    spec = Q.methane_minimal()
    pos = oracle.init_positions(spec, 8, seed=7)
    a = oracle.sweeps(spec, pos, 3, 0, 2, seed=99, step=0.3, threads=1)
    b = oracle.sweeps(spec, pos, 3, 0, 2, seed=99, step=0.3, threads=4)
    np.testing.assert_array_equal(a[0], b[0])
    assert a[1].sum() > 0


# ---------------------------------------------------------------------------
# Homogeneous electron gas (src/systems/heg.rs)
# ---------------------------------------------------------------------------
def test_heg_box_and_shells():
    """heg.rs:943-972: L = (4 pi N / 3)^(1/3) r_s; first k = 0, next six at 2 pi / L;
    27 orbitals per spin close the third shell."""
    spec = Q.electron_gas(54, 4.0)
    assert abs(spec.box_L - (4 * math.pi / 3 * 54) ** (1 / 3) * 4.0) < 1e-12
    kn = np.linalg.norm(spec.mo_coef, axis=1)
    assert kn[0] == 0.0
    np.testing.assert_allclose(kn[1:7], 2 * math.pi / spec.box_L, rtol=1e-14)
    shells = sorted(set(np.round(kn / (2 * math.pi / spec.box_L), 8)))
    assert shells == [0.0, 1.0, round(math.sqrt(2), 8), round(math.sqrt(3), 8)]


def test_heg_fourteen_electrons_and_cusp_amplitudes():
    """heg.rs:943-993: 14 electrons at r_s = 4 (7 per spin): L = (4 pi 14 / 3)^(1/3) r_s,
    k = 0 then six vectors of the first shell; the Jastrow amplitudes A_same = 0.5,
    A_anti = 0.25 (heg.rs:146-147)."""
    spec = Q.electron_gas(14, 4.0)
    assert abs(spec.box_L - (4 * math.pi / 3 * 14) ** (1 / 3) * 4.0) < 1e-10
    assert list(spec.spins).count(1) == 7 and list(spec.spins).count(-1) == 7
    kn = np.linalg.norm(spec.mo_coef, axis=1)
    assert len(kn) == 7 and kn[0] == 0.0
    np.testing.assert_allclose(kn[1:], 2 * math.pi / spec.box_L, rtol=1e-12)
    assert spec.jas[2] == 0.25 and spec.jas[3] == 0.5       # antiparallel, parallel


def test_heg_madelung_constant(oracle):
    """One electron in a cubic box with a neutralising background: the Ewald
    energy is -xi / (2 L) with the simple-cubic Madelung constant
    xi = 2.837297 (Nijboer & de Wette)."""
    spec = Q.electron_gas(n_elec=1, rs=3.0)
    e = oracle.heg_ewald(spec, np.array([[0.3, 1.7, 2.2]]))
    assert abs(e - (-2.837297479 / (2 * spec.box_L))) < 1e-8


@pytest.mark.parametrize("alphaL,kmax", [(4.0, 6), (4.0, 7), (6.0, 11), (7.0, 13)])
def test_heg_ewald_alpha_invariance(oracle, alphaL, kmax):
    """The one-component-plasma Ewald energy does not depend on the splitting
    parameter to 1e-8 Ha (the 54-electron workload's convergence target)."""
    spec = Q.electron_gas(54, 4.0)
    r = np.random.default_rng(3).uniform(0, spec.box_L, (54, 3))
    assert abs(oracle.heg_ewald(spec, r, 5.0, 8) - oracle.heg_ewald(spec, r, alphaL, kmax)) < 1e-8


def test_heg_local_energy_vs_fd(oracle):
    """Closed-shell Gamma-point determinants have a constant phase, so
    Re(lap psi / psi) = lap ln|psi| + |grad ln|psi||^2: the analytic gradient
    and Laplacian match central differences of ln|psi|."""
    spec = Q.electron_gas(54, 4.0)
    r = np.random.default_rng(5).uniform(0, spec.box_L, (54, 3))
    o = oracle.evaluate(spec, r)
    g, l = fd_grad_lap(oracle, spec, r, h=1e-4)
    np.testing.assert_allclose(o["grad"][0], g, rtol=1e-6, atol=1e-6 * np.abs(g).max())
    np.testing.assert_allclose(o["lap"][0], l, rtol=1e-4, atol=1e-4 * np.abs(l).max())


def test_heg_reference_quirks_differ(oracle):
    """The reference's Ewald (alpha = 5/L, |n_i| <= 7, no self or background
    term, -0.448 N / r_s) and cross term give a different local energy; both
    stay finite (heg.rs:1009-1030)."""
    r = np.random.default_rng(6).uniform(0, 24.0, (2, 54, 3))
    a = oracle.evaluate(Q.electron_gas(54, 4.0), r)["e_local"]
    b = oracle.evaluate(Q.electron_gas(54, 4.0, reference_quirks=True), r)["e_local"]
    assert np.all(np.isfinite(a)) and np.all(np.isfinite(b))
    assert np.all(np.abs(a - b) > 1e-3)


def test_heg_jastrow_gradient_antisymmetric(oracle):
    """heg.rs:1051-1063: two electrons, grad_1 u = -grad_2 u."""
    spec = Q.electron_gas(54, 4.0)
    r = np.random.default_rng(7).uniform(0, spec.box_L, (54, 3))
    o = oracle.evaluate(spec, r)
    assert np.linalg.norm(o["grad"][0].sum(axis=0)) < 1e-6 * np.abs(o["grad"]).max() * 54


@pytest.mark.parametrize("name", ["ch4_min", "ch4_gto", "c6h6"])
def test_el_derivatives_match_finite_differences(oracle, name):
    """The oracle's analytic dE_L/dp (Jastrow parameters and MO-rotation
    angles) against Richardson-extrapolated central differences of its E_L
    (steps 2h and h, h = 1e-4): 1e-6 relative.  Plain central differences at
    h = 1e-4 carry an O(h^2) truncation error of up to ~1e-4 relative for the
    rotation angles near a node, which the extrapolation removes."""
    import rust_qmc_gb300.systems as S
    spec = {"ch4_min": S.methane_minimal, "ch4_gto": S.methane_gto, "c6h6": S.benzene_minimal}[name]()
    p = np.asarray(spec.params(), dtype=np.float64)
    p[:8] = [1.3, 1.7, 0.45, 0.3, 1.9, 2.4, 0.8, 1.1]
    if len(p) > 8:
        p[8:] = [0.1, -0.2, 0.05, 0.3][: len(p) - 8]
    spec = spec.with_params(p)
    cfg = random_configs(spec, 3 if name == "c6h6" else 8, seed=3)
    a = oracle.el_derivatives(spec, cfg)
    f1 = oracle.el_derivatives_fd(spec, cfg, h=2e-4)
    f2 = oracle.el_derivatives_fd(spec, cfg, h=1e-4)
    fd = (4 * f2 - f1) / 3
    np.testing.assert_allclose(a, fd, rtol=1e-6, atol=1e-6 * np.abs(fd).max())


def test_benzene_gto_reference_checks(oracle):
    """The reference's own BenzeneGTO tests (src/systems/benzene.rs:871-1006)
    on benzene_gto: geometry (ring of radius 2.640, 120 degree angles, planar,
    C-H 2.042), 66 AOs and 21 MOs, V_nn in (180, 230), 21 + 21 electrons,
    psi finite at an initial configuration, analytic gradient against
    central differences, and the four reference log-derivatives (b_ee, b_en,
    a_anti, a_para at BenzeneGTO::new(2.0, 3.0)) against finite differences."""
    spec = Q.benzene_gto()
    R, Z = spec.nuc_pos, spec.nuc_charge
    C, H = R[Z == 6], R[Z == 1]
    for i in range(6):
        assert abs(np.linalg.norm(C[i]) - 2.640) < 1e-10
        assert abs(np.linalg.norm(C[i] - C[(i + 1) % 6]) - 2.640) < 0.01
        v1, v2 = C[(i + 5) % 6] - C[i], C[(i + 1) % 6] - C[i]
        assert abs(math.degrees(math.acos(v1 @ v2 / np.linalg.norm(v1) / np.linalg.norm(v2))) - 120.0) < 0.1
        assert abs(np.linalg.norm(C[i] - H[i]) - 2.042) < 0.01
    assert np.all(np.abs(R[:, 2]) < 1e-10)
    assert len(spec.ao_nuc) == 66 and spec.mo_coef.shape == (21, 66)
    assert 180.0 < spec.v_nn() < 230.0
    assert spec.n_elec == 42 and np.sum(np.asarray(spec.spins) > 0) == 21
    r = oracle.init_positions(spec, 2, seed=12)
    ev = oracle.evaluate(spec, r)
    assert np.all(np.isfinite(ev["logabs"])) and np.all(np.isfinite(ev["e_local"]))
    g, _ = fd_grad_lap(oracle, spec, r[0], h=1e-5)
    for i in (0, 10, 20, 30, 40):
        np.testing.assert_allclose(ev["grad"][0, i], g[i], rtol=1e-5, atol=1e-6 * (1 + np.abs(g[i]).max()))
    spec2 = Q.benzene_gto(2.0, 3.0)
    r2 = oracle.init_positions(spec2, 1, seed=13)
    O = oracle.log_derivatives(spec2, r2)[0]
    ref4 = [O[0] + O[1], O[4] + O[5], O[2], O[3]]
    p = Q.reference_params_from_general(spec2.params())
    h = 1e-5
    for k in range(4):
        pp, pm = list(p), list(p)
        pp[k] += h
        pm[k] -= h
        lp = oracle.evaluate(spec2.with_params(Q.jastrow3_params(*pp)), r2)["logabs"][0]
        lm = oracle.evaluate(spec2.with_params(Q.jastrow3_params(*pm)), r2)["logabs"][0]
        assert abs(ref4[k] - (lp - lm) / (2 * h)) <= 1e-6 * max(1.0, abs(ref4[k]))


def test_benzene_gto_mo_table_structure():
    """The hand-built MO table of src/systems/benzene.rs:262-470: core MOs on
    one carbon each, the pi MOs only on 2pz AOs, the C-H MOs touching one
    hydrogen each, and the ring MOs normalised over their phase patterns."""
    M = Q.benzene_gto().mo_coef
    for n in range(6):
        assert np.count_nonzero(M[n]) == 3 and M[n, 9 * n] == 0.9943
        nz = np.nonzero(M[9 + n])[0]
        assert set(nz[nz >= 54].tolist()) == {54 + 2 * n, 55 + 2 * n}
    pz = [9 * n + 4 for n in range(6)] + [9 * n + 8 for n in range(6)]
    for k in (15, 16, 17):
        assert set(np.nonzero(M[k])[0].tolist()) <= set(pz)
    assert np.all(M[15:18, [9 * n + 2 for n in range(6)]] == 0)

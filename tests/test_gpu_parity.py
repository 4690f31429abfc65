"""GPU parity of the CUDA walker path against the FP64 oracle, through the C ABI.

Tolerances (stated per test):
  * FP64 kernels vs oracle: 1e-10 relative on log|psi|, drift, Laplacian,
    E_L (absolute 1e-10 * max(1, |E_L|)).
  * FP32 working precision vs oracle: E_L measured by the FP64 refresh of
    FP32 walkers must be within 1e-6 Ha of the oracle at the same (float)
    configuration.
  * Trajectories: the counter-based Philox stream makes FP64 GPU sweeps and
    the oracle's reference-algorithm sweeps follow the same chain; positions
    agree to 1e-9 and accepted-move counts exactly.  A walker may leave the
    oracle's chain only where the oracle shows one of its acceptance
    decisions within 1e-9 (relative) of the threshold, the only place two
    FP64 evaluations that agree to ~1e-12 can decide differently.
  * Statistics: FP32+refine and FP64 energies agree within 4 combined
    standard errors (blocking errors, src/sampling/vmc.rs:166-188), with
    runs long enough that the combined error is a few mHa.
"""
import numpy as np
import pytest

import rust_qmc_gb300 as Q
from rust_qmc_gb300 import _lib as L
from tests.helpers import blocking_error, random_configs

pytestmark = pytest.mark.gpu

BUILDERS = {
    "h2": lambda: Q.h2_mo(),
    "li_ref": lambda: Q.lithium_atom(reference_quirks=True),
    "li_fixed": lambda: Q.lithium_atom(reference_quirks=False),
    "ch4_gto": lambda: Q.methane_gto(),
    "ch4_min": lambda: Q.methane_minimal(),
}


def rel(a, b):
    return np.max(np.abs(a - b) / np.maximum(1.0, np.abs(b)))


def assert_same_chain(got, want, margin, acc, acc_o, tol=1e-9):
    """Every walker of the device chain follows the oracle's chain, except a
    walker whose oracle run came within 1e-9 (relative) of an opposite
    acceptance decision; accepted counts agree exactly when all walkers do."""
    same = np.all(np.abs(got - want) < tol, axis=(1, 2))
    unexplained = ~same & (margin > 1e-9)
    assert not unexplained.any(), ("walkers off the oracle's chain", np.where(unexplained)[0],
                                   margin[unexplained])
    if same.all():
        assert acc == acc_o.sum(), (acc, acc_o.sum())
    return same


def assert_energies_agree(a, b, max_sigma):
    """Two runs of the same seed (FP64 and FP32+refine walkers from the same
    initial configurations and the same Philox stream) sample correlated
    chains; their per-measurement energy difference d_t = E_b,t - E_a,t has
    its own blocking error sigma_d, far below either run's.  Asserts
    |<d>| < 4 sigma_d with sigma_d below max_sigma (and at least 4 blocks),
    and |E_a - E_b| < 4 sigma_combined of the two runs' own errors."""
    d = np.asarray(b["energies"]) - np.asarray(a["energies"])
    sig_d, nb = blocking_error(d)
    assert nb >= 4 and 0 < sig_d < max_sigma, (sig_d, nb)
    assert abs(d.mean()) < 4 * sig_d, (d.mean(), sig_d)
    sig = np.hypot(a["error"], b["error"])
    if sig > 0:        # runs with fewer than two blocks of ceil(2 tau_int) report no error of their own
        assert abs(a["energy"] - b["energy"]) < 4 * sig, (a["energy"], b["energy"], sig)


@pytest.mark.parametrize("name", list(BUILDERS))
def test_eval_batch_fp64_matches_oracle(ctx, oracle, name):
    spec = BUILDERS[name]()
    sysh = Q.System(ctx, spec)
    cfg = random_configs(spec, 257, seed=1)
    g = sysh.eval_batch(cfg, L.QMC_FP64)
    o = oracle.evaluate(spec, cfg)
    assert np.array_equal(g["sign"], o["sign"])
    assert rel(g["logabs"], o["logabs"]) < 1e-10
    assert rel(g["grad"], o["grad"]) < 1e-10
    assert rel(g["lap"], o["lap"]) < 1e-10
    assert rel(g["e_local"], o["e_local"]) < 1e-10


@pytest.mark.parametrize("name", ["h2", "li_ref", "ch4_gto", "ch4_min"])
def test_eval_batch_fp32_close_to_oracle(ctx, oracle, name):
    """The single-precision evaluation used by moving walkers: ratios and
    drift to ~1e-4 relative (FP32 orbitals near carbon cores lose digits)."""
    spec = BUILDERS[name]()
    sysh = Q.System(ctx, spec)
    cfg = random_configs(spec, 128, seed=2).astype(np.float32).astype(np.float64)
    g = sysh.eval_batch(cfg, L.QMC_FP32_REFINE)
    o = oracle.evaluate(spec, cfg)
    assert np.mean(g["sign"] == o["sign"]) > 0.98
    ok = g["sign"] == o["sign"]
    assert np.median(np.abs(g["logabs"] - o["logabs"])[ok]) < 1e-4
    assert np.median(np.abs(g["e_local"] - o["e_local"]) / np.maximum(1, np.abs(o["e_local"]))) < 1e-3


@pytest.mark.parametrize("precision", [L.QMC_FP64, L.QMC_FP32_REFINE])
def test_init_matches_oracle(ctx, oracle, precision):
    spec = Q.methane_minimal()
    sysh = Q.System(ctx, spec)
    wk = Q.Walkers(sysh, 300, precision)
    wk.init(seed=1234)
    got = wk.get_positions()
    want = oracle.init_positions(spec, 300, seed=1234)
    if precision == L.QMC_FP32_REFINE:
        want = want.astype(np.float32).astype(np.float64)
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-12 if precision == L.QMC_FP64 else 1e-6)


@pytest.mark.parametrize("name", ["ch4_min", "ch4_gto", "li_ref", "h2"])
def test_fp32_walkers_refresh_energy_within_1e6(ctx, oracle, name):
    """FP32 walkers after sweeps: the refresh E_L (float-float arithmetic,
    48-bit significand) equals the oracle's FP64 E_L of the same (float)
    configuration to <= 1e-6 Ha -- the error budget -- and in fact to
    FP64-class accuracy: 1e-9 relative on E_L, 1e-10 on log|psi|."""
    spec = BUILDERS[name]()
    sysh = Q.System(ctx, spec)
    W = 512
    wk = Q.Walkers(sysh, W, L.QMC_FP32_REFINE)
    wk.init(seed=77)
    wk.refresh()
    wk.sweep(L.QMC_MOVE_ONE_GAUSS, 16, 0, seed=5, step=0.3)
    _, el = wk.refresh(want_energies=True)
    logabs, sign, _ = wk.state()
    pos = wk.get_positions()
    o = oracle.evaluate(spec, pos)
    err = np.abs(el - o["e_local"])
    assert np.max(err) <= 1e-6, np.max(err)
    assert rel(el, o["e_local"]) < 1e-9
    assert rel(logabs, o["logabs"]) < 1e-10
    assert np.array_equal(sign, o["sign"])


@pytest.mark.parametrize("name,move", [("ch4_min", L.QMC_MOVE_ONE_GAUSS), ("ch4_min", L.QMC_MOVE_ONE_DRIFT),
                                       ("ch4_gto", L.QMC_MOVE_ONE_DRIFT), ("li_ref", L.QMC_MOVE_ONE_GAUSS),
                                       ("li_ref", L.QMC_MOVE_ONE_DRIFT), ("h2", L.QMC_MOVE_ONE_GAUSS)])
def test_fp64_single_electron_trajectory_matches_oracle(ctx, oracle, name, move):
    spec = BUILDERS[name]()
    sysh = Q.System(ctx, spec)
    W, n = 256, 4
    wk = Q.Walkers(sysh, W, L.QMC_FP64)
    wk.init(seed=31)
    wk.refresh()
    pos0 = wk.get_positions()
    acc = wk.sweep(move, n, 10, seed=4242, step=0.3, tau=0.02, max_drift=1.0)
    got = wk.get_positions()
    want, acc_o, _, mg = oracle.sweeps(spec, pos0, n, 10, move, 4242, step=0.3, tau=0.02, max_drift=1.0,
                                       want_energy=False, want_margin=True)
    assert_same_chain(got, want, mg, acc, acc_o)
    assert acc > 0


@pytest.mark.parametrize("move", [L.QMC_MOVE_ALL_BOX, L.QMC_MOVE_ALL_GAUSS])
def test_fp64_all_electron_trajectory_matches_oracle(ctx, oracle, move):
    spec = Q.h2_mo()
    sysh = Q.System(ctx, spec)
    W, n = 128, 20
    wk = Q.Walkers(sysh, W, L.QMC_FP64)
    wk.init(seed=8)
    wk.refresh()
    pos0 = wk.get_positions()
    acc = wk.sweep(move, n, 0, seed=99, step=1.0)
    got = wk.get_positions()
    want, acc_o, el_o, mg = oracle.sweeps(spec, pos0, n, 0, move, 99, step=1.0, want_margin=True)
    same = assert_same_chain(got, want, mg, acc, acc_o)
    _, _, el = wk.state()
    np.testing.assert_allclose(el[same], el_o[same], rtol=1e-10, atol=1e-10)


def test_refresh_restores_inverse_after_long_fp32_run(ctx, oracle):
    """Sherman-Morrison drift in FP32 over 64 sweeps stays small enough that
    acceptance matches the FP64 chain statistically, and the refresh E_L is
    the oracle's."""
    spec = Q.methane_minimal()
    sysh = Q.System(ctx, spec)
    W = 4096
    wk = Q.Walkers(sysh, W, L.QMC_FP32_REFINE)
    wk.init(seed=3)
    wk.refresh()
    acc = wk.sweep(L.QMC_MOVE_ONE_GAUSS, 64, 0, seed=17, step=0.3)
    assert 0.2 < acc / (64 * 10 * W) < 0.95
    s, el = wk.refresh(want_energies=True)
    assert np.all(np.isfinite(el))
    assert abs(s - el.sum()) < 1e-6 * max(1.0, abs(s))
    assert wk.status() & 1 == 0


@pytest.mark.parametrize("name", ["ch4_min", "ch4_gto"])
def test_logderiv_batch_matches_oracle(ctx, oracle, name):
    spec = BUILDERS[name]()
    if name == "ch4_min":
        spec = spec.with_params(np.concatenate([spec.jas, [0.1, -0.2, 0.05, 0.3]]))
    sysh = Q.System(ctx, spec)
    cfg = random_configs(spec, 1000, seed=6)
    O, E, S, f, em = sysh.logderiv_batch(cfg, sums=True)
    Oo = oracle.log_derivatives(spec, cfg)
    Eo = oracle.evaluate(spec, cfg)["e_local"]
    assert rel(O, Oo) < 1e-10
    assert rel(E, Eo) < 1e-10
    n = len(E)
    Om = Oo.mean(0)
    S_ref = Oo.T @ Oo / n - np.outer(Om, Om)
    f_ref = (Eo[:, None] * Oo).mean(0) - Eo.mean() * Om
    np.testing.assert_allclose(S, S_ref, rtol=1e-9, atol=1e-9 * np.abs(S_ref).max())
    np.testing.assert_allclose(f, f_ref, rtol=1e-8, atol=1e-8 * np.abs(f_ref).max())
    assert abs(em - Eo.mean()) < 1e-9 * max(1, abs(em))


@pytest.mark.parametrize("name", ["h2", "ch4_min", "ch4_gto"])
def test_forces_match_oracle_and_fd(ctx, oracle, name):
    spec = BUILDERS[name]()
    sysh = Q.System(ctx, spec)
    cfg = random_configs(spec, 64, seed=12)
    F, Om = sysh.forces_batch(cfg)
    Fo, Omo = oracle.forces(spec, cfg)
    assert rel(F, Fo) < 1e-10
    assert rel(Om, Omo) < 1e-10
    fd = oracle.nuclear_gradient_fd(spec, cfg[:8], h=1e-5)
    np.testing.assert_allclose(Om[:8], fd, rtol=1e-5, atol=1e-6)


def test_benzene_hf_force_matches_oracle(ctx, oracle):
    """BenzeneGTO's ForceCalculator (src/systems/benzene.rs:811-858): the
    Hellmann-Feynman force per configuration; it has no wave-function nuclear
    gradient (the trait's unimplemented default), so asking for one fails."""
    spec = Q.benzene_minimal()
    sysh = Q.System(ctx, spec)
    cfg = random_configs(spec, 37, seed=13)
    F, Om = sysh.forces_batch(cfg, omega=False)
    assert Om is None
    Fo, _ = oracle.forces(spec, cfg)
    assert rel(F, Fo) < 1e-12
    with pytest.raises(Q.QMCError):
        sysh.forces_batch(cfg[:2])


def test_trait_surface_single_configuration(ctx, oracle):
    """MultiWfn/EnergyCalculator/OptimizableWfn/ForceCalculator methods with
    the reference's value conventions (psi, grad psi, lap psi)."""
    spec = Q.methane_gto()
    sysh = Q.System(ctx, spec)
    r = random_configs(spec, 1, seed=40)[0]
    o = oracle.evaluate(spec, r)
    psi = o["sign"][0] * np.exp(o["logabs"][0])
    assert abs(sysh.evaluate(r) - psi) <= 1e-10 * abs(psi)
    np.testing.assert_allclose(sysh.derivative(r), o["grad"][0] * psi, rtol=1e-9, atol=1e-12 * abs(psi))
    np.testing.assert_allclose(sysh.laplacian(r), o["lap"][0] * psi, rtol=1e-9, atol=1e-12 * abs(psi))
    assert abs(sysh.local_energy(r) - o["e_local"][0]) < 1e-9
    p = sysh.get_params()
    p2 = p.copy()
    p2[0] += 0.1
    sysh.set_params(p2)
    assert np.allclose(sysh.get_params(), p2)
    assert abs(sysh.local_energy(r) - oracle.evaluate(spec.with_params(p2), r)["e_local"][0]) < 1e-9
    R = spec.nuc_pos.copy()
    R[1] += 0.05
    sysh.set_nuclei(R)
    o2 = oracle.evaluate(spec.with_params(p2).with_nuclei(R), r)
    assert abs(sysh.local_energy(r) - o2["e_local"][0]) < 1e-9
    with pytest.raises(Q.QMCError):
        sysh.set_params(np.zeros(3))


def test_vmc_run_h2_box_moves(ctx):
    """MCMCSimulation on H2 (all-electron uniform box of 1.0 bohr): energy
    in the LCAO-Jastrow range and the error bar from blocking."""
    sysh = Q.System(ctx, Q.h2_mo())
    r = Q.vmc_run(sysh, n_walkers=1024, n_steps=400, n_burnin=100, move_kind=L.QMC_MOVE_ALL_BOX, step=1.0,
                  seed=5)
    assert -1.20 < r["energy"] < -1.10, r
    assert 0 < r["error"] < 0.01
    assert 0.3 < r["acceptance_rate"] < 0.95
    assert r["n_samples"] == 400


@pytest.mark.parametrize("name", ["ch4_min", "c6h6", "c6h6_gto", "heg"])
def test_vmc_run_precisions_agree(ctx, name):
    """FP32+refine and FP64 chains give statistically indistinguishable
    energies: the paired energy difference of two same-seed runs within 4
    of its blocking errors, no slack beyond the error bars.  The error caps
    follow the E_L variance of each trial function (the synthetic benzene's
    seeded MOs give E_L a standard deviation near 50 Ha; the electron gas
    decorrelates over hundreds of sweeps): 2 mHa for CH4, 10 mHa for the
    benzenes, 20 mHa for the electron gas."""
    spec = {"ch4_min": Q.methane_minimal, "c6h6": Q.benzene_minimal, "c6h6_gto": Q.benzene_gto,
            "heg": Q.electron_gas}[name]()
    sysh = Q.System(ctx, spec)
    W, n, burn, step, cap = {"ch4_min": (65536, 2048, 128, 0.3, 2e-3), "c6h6": (8192, 1024, 64, 0.3, 10e-3),
                             "c6h6_gto": (8192, 1024, 64, 0.3, 10e-3), "heg": (2048, 4096, 64, 0.5, 20e-3)}[name]
    res = {}
    for prec in (L.QMC_FP64, L.QMC_FP32_REFINE):
        res[prec] = Q.vmc_run(sysh, n_walkers=W, n_steps=n, n_burnin=burn, move_kind=L.QMC_MOVE_ONE_GAUSS,
                              step=step, precision=prec, refresh_every=8, seed=11)
    assert_energies_agree(res[L.QMC_FP64], res[L.QMC_FP32_REFINE], cap)


@pytest.mark.parametrize("name,fixed_node,refdiff", [("h2", True, False), ("ch4_min", True, False),
                                                     ("li_ref", False, True)])
def test_fp64_dmc_population_matches_oracle(ctx, oracle, name, fixed_node, refdiff):
    """IS-DMC branching + compaction: the FP64 device population follows the
    oracle's reference-algorithm DMC step for step (same Philox stream,
    order-stable copies), so populations and mean energies agree."""
    spec = BUILDERS[name]()
    sysh = Q.System(ctx, spec)
    target, n_steps, tau = 48, 6, 0.02
    wk = Q.Walkers(sysh, target, L.QMC_FP64, capacity=4 * target)
    wk.init(seed=21)
    e_sum = wk.refresh()
    e_ref = e_sum / target
    pos0 = wk.get_positions()
    pops, ens = [], []
    er = e_ref
    for t in range(n_steps):
        n, em = wk.dmc_step(tau, er, seed=77, step=t, fixed_node=fixed_node, reference_diffusion=refdiff)
        assert n > 0
        pops.append(n)
        ens.append(em)
        er = em - 0.5 * np.log(n / target) / tau
    _, pops_o, ens_o, er_o = oracle.dmc(spec, pos0, n_steps, tau, e_ref, target, 77, fixed_node=fixed_node,
                                        reference_diffusion=refdiff)
    assert list(pops) == list(pops_o)
    np.testing.assert_allclose(ens, ens_o, rtol=1e-9, atol=1e-9)
    got = wk.get_positions()
    want, _, _, _ = oracle.dmc(spec, pos0, n_steps, tau, e_ref, target, 77, fixed_node=fixed_node,
                               reference_diffusion=refdiff)
    np.testing.assert_allclose(got, want, atol=1e-8)


def test_dmc_run_h2_energy(ctx):
    """DMC of H2 (nodeless ground state) with Hartree-unit diffusion reaches
    the exact -1.1745 Ha within statistical, time-step and population bias;
    the reference's diffusion (variance 2 tau with branching at tau) settles
    markedly higher, which is why it is behind a flag."""
    sysh = Q.System(ctx, Q.h2_mo())
    d = Q.dmc_run(sysh, n_walkers=4096, n_steps=800, n_burnin=800, tau=0.005, seed=3)
    r = Q.dmc_run(sysh, n_walkers=4096, n_steps=800, n_burnin=800, tau=0.005, seed=3, reference_diffusion=True)
    v = Q.vmc_run(sysh, n_walkers=2048, n_steps=400, n_burnin=100, move_kind=L.QMC_MOVE_ALL_BOX, step=1.0, seed=4)
    assert abs(d["energy"] - (-1.1745)) < 0.004 + 4 * d["error"], d
    assert r["energy"] > d["energy"] + 0.005, (r, d)
    assert d["energy"] < v["energy"] + 3 * (d["error"] + v["error"])
    assert 3000 < d["avg_population"] < 5500
    assert 0.9 < d["acceptance_rate"] <= 1.0


@pytest.mark.parametrize("name", ["h2", "c6h6_gto"])
def test_dmc_precisions_agree(ctx, name):
    """FP32+refine and FP64 DMC populations (same seed) give statistically
    indistinguishable energies, no slack beyond the error bars; the FP32
    form measures E_L in FP64-class arithmetic every 8 steps.  H2 runs the
    reference's branching; the reference's benzene runs with the branching
    energy clamped to E_ref +- 2/sqrt(tau) (qmc_run_params.branch_cut), which
    keeps the population finite where its nodal E_L divergences otherwise
    explode it.  Branching decorrelates the two populations within a few
    steps, so the paired difference has about the two runs' combined error:
    2 mHa for H2, 0.25 Ha for benzene (a mixed estimate of -228.6 Ha from 2048
    walkers; 4e-4 relative)."""
    spec = {"h2": Q.h2_mo, "c6h6_gto": Q.benzene_gto}[name]()
    sysh = Q.System(ctx, spec)
    W, n, burn, cap, cut = {"h2": (8192, 1000, 200, 2e-3, 0.0),
                            "c6h6_gto": (2048, 400, 200, 0.25, 2.0 / np.sqrt(0.005))}[name]
    r = {}
    for prec in (L.QMC_FP64, L.QMC_FP32_REFINE):
        r[prec] = Q.dmc_run(sysh, n_walkers=W, n_steps=n, n_burnin=burn, tau=0.005, precision=prec,
                            refresh_every=8, seed=5, branch_cut=cut)
    a, b = r[L.QMC_FP64], r[L.QMC_FP32_REFINE]
    assert np.isfinite(a["energy"]) and np.isfinite(b["energy"])
    assert 0.5 * W < a["avg_population"] < 2 * W and 0.5 * W < b["avg_population"] < 2 * W
    assert_energies_agree(a, b, cap)


def test_fp64_dmc_population_with_branch_cut_matches_oracle(ctx, oracle):
    """The clamped branching (branch_cut) on the device follows the oracle's
    DMC with the same clamp population for population."""
    spec = Q.methane_minimal()
    sysh = Q.System(ctx, spec)
    target, n_steps, tau, cut = 48, 6, 0.02, 1.5
    wk = Q.Walkers(sysh, target, L.QMC_FP64, capacity=4 * target)
    wk.init(seed=21)
    e_ref = wk.refresh() / target
    pos0 = wk.get_positions()
    pops, ens, er = [], [], e_ref
    for t in range(n_steps):
        n, em = wk.dmc_step(tau, er, seed=77, step=t, fixed_node=True, branch_cut=cut)
        pops.append(n)
        ens.append(em)
        er = em - 0.5 * np.log(n / target) / tau
    _, pops_o, ens_o, _ = oracle.dmc(spec, pos0, n_steps, tau, e_ref, target, 77, fixed_node=True, branch_cut=cut)
    assert list(pops) == list(pops_o)
    np.testing.assert_allclose(ens, ens_o, rtol=1e-9, atol=1e-9)


# ---------------------------------------------------------------------------
# Benzene (warp-per-walker kernels)
# ---------------------------------------------------------------------------
def test_benzene_eval_fp64_matches_oracle(ctx, oracle):
    spec = Q.benzene_minimal()
    sysh = Q.System(ctx, spec)
    cfg = random_configs(spec, 37, seed=4)
    g = sysh.eval_batch(cfg, L.QMC_FP64)
    o = oracle.evaluate(spec, cfg)
    assert np.array_equal(g["sign"], o["sign"])
    assert rel(g["logabs"], o["logabs"]) < 1e-10
    assert rel(g["grad"], o["grad"]) < 1e-9
    assert rel(g["lap"], o["lap"]) < 1e-9
    assert rel(g["e_local"], o["e_local"]) < 1e-10


def test_benzene_log_derivatives_and_sr_sums(ctx, oracle):
    """BenzeneGTO's OptimizableWfn (src/systems/benzene.rs:726-756) on the
    device: the eight Jastrow log-derivatives per configuration, E_L from the
    FP64 refresh, and the SR sums S, f over the batch."""
    spec = Q.benzene_minimal()
    sysh = Q.System(ctx, spec)
    cfg = random_configs(spec, 96, seed=15)
    O, E, S, f, em = sysh.logderiv_batch(cfg, sums=True)
    Oo = oracle.log_derivatives(spec, cfg)
    Eo = oracle.evaluate(spec, cfg)["e_local"]
    assert O.shape == (96, 8)
    assert rel(O, Oo) < 1e-10
    assert rel(E, Eo) < 1e-9
    n = len(E)
    Om = Oo.mean(0)
    S_ref = Oo.T @ Oo / n - np.outer(Om, Om)
    f_ref = (Eo[:, None] * Oo).mean(0) - Eo.mean() * Om
    np.testing.assert_allclose(S, S_ref, rtol=1e-8, atol=1e-8 * np.abs(S_ref).max())
    np.testing.assert_allclose(f, f_ref, rtol=1e-7, atol=1e-7 * np.abs(f_ref).max())
    assert abs(em - Eo.mean()) < 1e-9 * max(1.0, np.abs(Eo).mean())


@pytest.mark.parametrize("move", [L.QMC_MOVE_ONE_GAUSS, L.QMC_MOVE_ONE_DRIFT])
def test_benzene_fp64_trajectory_matches_oracle(ctx, oracle, move):
    spec = Q.benzene_minimal()
    sysh = Q.System(ctx, spec)
    W, n = 256, 4
    wk = Q.Walkers(sysh, W, L.QMC_FP64)
    wk.init(seed=5)
    wk.refresh()
    pos0 = wk.get_positions()
    acc = wk.sweep(move, n, 3, seed=606, step=0.3, tau=0.005, max_drift=1.0)
    got = wk.get_positions()
    want, acc_o, _, mg = oracle.sweeps(spec, pos0, n, 3, move, 606, step=0.3, tau=0.005, max_drift=1.0,
                                       want_energy=False, want_margin=True)
    assert_same_chain(got, want, mg, acc, acc_o)


def test_benzene_fp32_refresh_energy_within_1e6(ctx, oracle):
    spec = Q.benzene_minimal()
    sysh = Q.System(ctx, spec)
    W = 64
    wk = Q.Walkers(sysh, W, L.QMC_FP32_REFINE)
    wk.init(seed=9)
    wk.refresh()
    acc = wk.sweep(L.QMC_MOVE_ONE_GAUSS, 8, 0, seed=10, step=0.3)
    assert acc > 0
    _, el = wk.refresh(want_energies=True)
    o = oracle.evaluate(spec, wk.get_positions())
    assert np.max(np.abs(el - o["e_local"])) <= 1e-6


def test_benzene_fp64_dmc_matches_oracle(ctx, oracle):
    spec = Q.benzene_minimal()
    sysh = Q.System(ctx, spec)
    target, n_steps, tau = 8, 2, 0.005
    wk = Q.Walkers(sysh, target, L.QMC_FP64, capacity=4 * target)
    wk.init(seed=12)
    e_ref = wk.refresh() / target
    pos0 = wk.get_positions()
    pops, ens, er = [], [], e_ref
    for t in range(n_steps):
        n, em = wk.dmc_step(tau, er, seed=13, step=t, fixed_node=True)
        pops.append(n)
        ens.append(em)
        er = em - 0.5 * np.log(n / target) / tau
    _, pops_o, ens_o, _ = oracle.dmc(spec, pos0, n_steps, tau, e_ref, target, 13, fixed_node=True)
    assert list(pops) == list(pops_o)
    np.testing.assert_allclose(ens, ens_o, rtol=1e-9, atol=1e-8)


# ---------------------------------------------------------------------------
# Periodic electron gas (complex plane-wave determinants, Ewald)
# ---------------------------------------------------------------------------
HEG_BUILDERS = {"heg": lambda: Q.electron_gas(), "heg_ref": lambda: Q.electron_gas(reference_quirks=True),
                "heg_twist": lambda: Q.electron_gas(twist=(0.25, -0.25, 0.25)),
                "heg_pade_twist": lambda: Q.electron_gas(form="pade", twist=(1.0 / 3.0, 0.0, -1.0 / 3.0)),
                "heg_yukawa": lambda: Q.electron_gas(form="yukawa")}


@pytest.mark.parametrize("name", list(HEG_BUILDERS))
def test_heg_eval_fp64_matches_oracle(ctx, oracle, name):
    spec = HEG_BUILDERS[name]()
    sysh = Q.System(ctx, spec)
    cfg = np.random.default_rng(8).uniform(0, spec.box_L, (9, 54, 3))
    g = sysh.eval_batch(cfg, L.QMC_FP64)
    o = oracle.evaluate(spec, cfg)
    assert rel(g["logabs"], o["logabs"]) < 1e-10
    assert rel(g["grad"], o["grad"]) < 1e-9
    assert rel(g["lap"], o["lap"]) < 1e-9
    # the real-space Ewald images beyond L/2 (each term < 3e-5 Ha) are summed
    # in FP32 on the device: E_L agrees to a few 1e-9 Ha absolute (the same
    # error for every Jastrow form), far inside the 1e-6 Ha budget
    assert np.max(np.abs(g["e_local"] - o["e_local"])) < 1e-8


@pytest.mark.parametrize("move", [L.QMC_MOVE_ONE_GAUSS, L.QMC_MOVE_ONE_DRIFT])
def test_heg_fp64_trajectory_matches_oracle(ctx, oracle, move):
    spec = Q.electron_gas()
    sysh = Q.System(ctx, spec)
    W, n = 256, 4
    wk = Q.Walkers(sysh, W, L.QMC_FP64)
    wk.init(seed=15)
    wk.refresh()
    pos0 = wk.get_positions()
    init = oracle.init_positions(spec, W, seed=15)
    np.testing.assert_allclose(pos0, init, atol=1e-12)
    acc = wk.sweep(move, n, 2, seed=616, step=1.0, tau=0.05, max_drift=1.0)
    got = wk.get_positions()
    want, acc_o, _, mg = oracle.sweeps(spec, pos0, n, 2, move, 616, step=1.0, tau=0.05, max_drift=1.0,
                                       want_energy=False, want_margin=True)
    assert_same_chain(got, want, mg, acc, acc_o, tol=1e-8)


def test_heg_fp32_refresh_energy_within_1e6(ctx, oracle):
    spec = Q.electron_gas()
    sysh = Q.System(ctx, spec)
    wk = Q.Walkers(sysh, 32, L.QMC_FP32_REFINE)
    wk.init(seed=17)
    wk.refresh()
    acc = wk.sweep(L.QMC_MOVE_ONE_GAUSS, 4, 0, seed=18, step=1.0)
    assert acc > 0
    _, el = wk.refresh(want_energies=True)
    o = oracle.evaluate(spec, wk.get_positions())
    assert np.max(np.abs(el - o["e_local"])) <= 1e-6


def test_handles_release_in_any_order(qmc_lib):
    """Parent handles destroyed before their children: the walker set keeps
    working and the deferred release frees everything when it goes."""
    c2 = Q.Context(0)
    sysh = Q.System(c2, Q.h2_mo())
    wk = Q.Walkers(sysh, 64, L.QMC_FP64)
    wk.init(seed=5)
    e0 = wk.refresh()
    assert qmc_lib.qmc_destroy(c2.h) == L.QMC_OK
    c2.h = None
    assert qmc_lib.qmc_system_destroy(sysh.h) == L.QMC_OK
    sysh.h = None
    wk.sweep(L.QMC_MOVE_ONE_GAUSS, 4, 0, seed=5, step=0.5)
    e1 = wk.refresh()
    assert np.isfinite(e0) and np.isfinite(e1) and e1 != e0
    assert qmc_lib.qmc_walkers_destroy(wk.h) == L.QMC_OK
    wk.h = None


@pytest.mark.parametrize("name", ["h2", "li_ref", "ch4_min"])
def test_ratio_batch_matches_oracle(ctx, oracle, name):
    """qmc_ratio_batch: psi ratio of a single-electron move and the drift at
    the moved configuration, against the oracle's two evaluations (1e-10)."""
    spec = BUILDERS[name]()
    sysh = Q.System(ctx, spec)
    cfg = random_configs(spec, 33, seed=11)
    rng = np.random.default_rng(12)
    for e in range(spec.n_elec):
        r_new = cfg[:, e, :] + 0.3 * rng.standard_normal((cfg.shape[0], 3))
        ratio, grad = sysh.ratio_batch(cfg, e, r_new)
        moved = cfg.copy()
        moved[:, e, :] = r_new
        o0, o1 = oracle.evaluate(spec, cfg), oracle.evaluate(spec, moved)
        want = o0["sign"] * o1["sign"] * np.exp(o1["logabs"] - o0["logabs"])
        assert rel(ratio, want) < 1e-10
        assert rel(grad, o1["grad"][:, e, :]) < 1e-10


@pytest.mark.parametrize("name", ["h2", "li_ref", "ch4_min", "c6h6", "heg"])
def test_refresh_energy_sum_matches_walker_energies(ctx, name):
    """The compensated E_L sum returned by a refresh equals the sum of the
    per-walker energies, for every kernel family and enough walkers that the
    warp-per-walker kernels launch hundreds of blocks."""
    builders = dict(BUILDERS, c6h6=lambda: Q.benzene_minimal(), heg=lambda: Q.electron_gas())
    sysh = Q.System(ctx, builders[name]())
    for prec in (L.QMC_FP32_REFINE, L.QMC_FP64):
        wk = Q.Walkers(sysh, 512, prec)
        wk.init(seed=19)
        e_sum, el = wk.refresh(want_energies=True)
        assert np.all(np.isfinite(el))
        assert abs(e_sum - el.sum()) <= 1e-12 * max(1.0, abs(el).sum())
        wk.close()


@pytest.mark.parametrize("prec", [L.QMC_FP32_REFINE, L.QMC_FP64])
def test_benzene_refresh_block_shapes_agree(ctx, prec):
    """The benzene refresh picks 4 or 8 walkers per block by timing both on
    its first call of 1024+ walkers; both shapes compute each walker alike,
    so the walker state after the tuning call equals the state after a later
    call with the chosen shape, bit for bit."""
    sysh = Q.System(ctx, Q.benzene_minimal())
    wk = Q.Walkers(sysh, 2048, prec)
    wk.init(seed=23)
    e1, el1 = wk.refresh(want_energies=True)
    la1, sg1, _ = wk.state()
    e2, el2 = wk.refresh(want_energies=True)
    la2, sg2, _ = wk.state()
    assert np.array_equal(el1, el2) and np.array_equal(la1, la2) and np.array_equal(sg1, sg2)
    assert abs(e1 - e2) <= 1e-12 * abs(el1).sum()
    assert abs(e2 - el2.sum()) <= 1e-12 * abs(el2).sum()


@pytest.mark.parametrize("name", ["h2", "li_ref", "ch4_min", "ch4_gto", "c6h6", "heg"])
@pytest.mark.parametrize("prec", [L.QMC_FP32_REFINE, L.QMC_FP64])
def test_rebuild_inverse_matches_refresh(ctx, name, prec):
    """qmc_walkers_rebuild_inverse leaves the walker state a full refresh
    leaves (log|psi| and sign bit for bit), and a Gaussian sweep after it
    follows the same trajectory as a sweep after the full refresh."""
    builders = dict(BUILDERS, c6h6=lambda: Q.benzene_minimal(), heg=lambda: Q.electron_gas())
    sysh = Q.System(ctx, builders[name]())
    W = 256
    src = Q.Walkers(sysh, W, prec)
    src.init(seed=41)
    pos = src.get_positions()
    src.close()
    out = []
    for rebuild in (False, True):
        wk = Q.Walkers(sysh, W, prec)
        wk.set_positions(pos)
        if rebuild:
            wk.rebuild_inverse()
        else:
            wk.refresh()
        la, sg, _ = wk.state()
        wk.sweep(L.QMC_MOVE_ONE_GAUSS, 4, 7, seed=5, step=0.3, count=False)
        out.append((la, sg, wk.get_positions(), wk.status()))
        wk.close()
    (la0, sg0, p0, f0), (la1, sg1, p1, f1) = out
    assert np.all(np.isfinite(la0))
    assert np.array_equal(la0, la1) and np.array_equal(sg0, sg1)
    assert np.array_equal(p0, p1)
    assert f0 == 0 and f1 == 0


@pytest.mark.parametrize("name", ["h2", "li_ref", "ch4_min", "ch4_gto"])
def test_fp64_gaussian_sweeps_ragged_walker_count(ctx, oracle, name):
    """Gaussian single-electron sweeps of 97 walkers (a partial last block of
    the 64-walker sweep blocks, with their shared-memory pair caches) follow
    the oracle's chains like full blocks do."""
    spec = BUILDERS[name]()
    sysh = Q.System(ctx, spec)
    W, n = 97, 3
    wk = Q.Walkers(sysh, W, L.QMC_FP64)
    wk.init(seed=57)
    wk.refresh()
    pos0 = wk.get_positions()
    acc = wk.sweep(L.QMC_MOVE_ONE_GAUSS, n, 3, seed=777, step=0.3)
    got = wk.get_positions()
    want, acc_o, _, mg = oracle.sweeps(spec, pos0, n, 3, L.QMC_MOVE_ONE_GAUSS, 777, step=0.3, want_energy=False,
                                       want_margin=True)
    assert_same_chain(got, want, mg, acc, acc_o)      # includes the 33 walkers of the partial block


def benzene_distinct():
    """Benzene with every Jastrow parameter distinct (b_anti != b_para,
    a_anti != a_para, B_C != B_H, A_C != A_H), so that a swap of spin class or
    species anywhere on the device changes the result."""
    spec = Q.benzene_minimal()
    return spec.with_params(np.array([1.3, 1.7, 0.45, 0.3, 1.9, 2.4, 0.8, 1.1]))


def test_benzene_distinct_parameters_eval_and_sr(ctx, oracle):
    spec = benzene_distinct()
    sysh = Q.System(ctx, spec)
    cfg = random_configs(spec, 40, seed=44)
    g = sysh.eval_batch(cfg, L.QMC_FP64)
    o = oracle.evaluate(spec, cfg)
    assert np.array_equal(g["sign"], o["sign"])
    assert rel(g["logabs"], o["logabs"]) < 1e-10
    assert rel(g["grad"], o["grad"]) < 1e-9
    assert rel(g["lap"], o["lap"]) < 1e-9
    assert rel(g["e_local"], o["e_local"]) < 1e-10
    O, E, S, f, em = sysh.logderiv_batch(cfg, sums=True)
    Oo = oracle.log_derivatives(spec, cfg)
    assert rel(O, Oo) < 1e-10
    Om = Oo.mean(0)
    np.testing.assert_allclose(S, Oo.T @ Oo / len(E) - np.outer(Om, Om), rtol=1e-8, atol=1e-8 * np.abs(S).max())


@pytest.mark.parametrize("move", [L.QMC_MOVE_ONE_GAUSS, L.QMC_MOVE_ONE_DRIFT])
def test_benzene_distinct_parameters_trajectory(ctx, oracle, move):
    spec = benzene_distinct()
    sysh = Q.System(ctx, spec)
    W, n = 256, 4
    wk = Q.Walkers(sysh, W, L.QMC_FP64)
    wk.init(seed=46)
    wk.refresh()
    pos0 = wk.get_positions()
    acc = wk.sweep(move, n, 5, seed=808, step=0.3, tau=0.005, max_drift=1.0)
    got = wk.get_positions()
    want, acc_o, _, mg = oracle.sweeps(spec, pos0, n, 5, move, 808, step=0.3, tau=0.005, max_drift=1.0,
                                       want_energy=False, want_margin=True)
    assert_same_chain(got, want, mg, acc, acc_o)


def test_benzene_distinct_parameters_fp32_refresh(ctx, oracle):
    spec = benzene_distinct()
    sysh = Q.System(ctx, spec)
    wk = Q.Walkers(sysh, 256, L.QMC_FP32_REFINE)
    wk.init(seed=47)
    wk.refresh()
    assert wk.sweep(L.QMC_MOVE_ONE_GAUSS, 8, 0, seed=48, step=0.3) > 0
    _, el = wk.refresh(want_energies=True)
    la, sg, _ = wk.state()
    o = oracle.evaluate(spec, wk.get_positions())
    assert np.max(np.abs(el - o["e_local"])) <= 1e-6
    assert rel(la, o["logabs"]) < 1e-10
    assert np.array_equal(sg, o["sign"])


@pytest.mark.parametrize("name", ["ch4_min", "c6h6", "heg"])
@pytest.mark.parametrize("move", [L.QMC_MOVE_ONE_GAUSS, L.QMC_MOVE_ONE_DRIFT])
def test_fp32_sweep_decisions_match_oracle(ctx, oracle, name, move):
    """Per-configuration check of the FP32 moving path: FP32 walkers and the
    oracle's FP64 reference algorithm start from the same (float-valued)
    configurations and draw the same proposals.  After one sweep every walker
    whose oracle run kept each acceptance decision more than 1e-3 (relative)
    away from its threshold must have taken exactly the oracle's decisions,
    i.e. the FP32 ratio psi'/psi is within 1e-3 of the FP64 one at every such
    proposal, and its positions agree to 2e-5 bohr.  Drift-diffusion moves
    carry the FP32 drift into the proposal and the Green's-function factor:
    there the band is 1e-2 and positions agree to 2e-4 bohr, which bounds the
    FP32 drift error by 2e-4 / (2 tau) per accepted move (5e-3 at tau = 0.02,
    2e-3 at 0.05 for the electron gas).  The few walkers with a decision
    inside the band may differ, and for drift moves up to 2 % more: close to
    a node the FP32 drift loses its relative accuracy."""
    spec = {"ch4_min": Q.methane_minimal, "c6h6": Q.benzene_minimal, "heg": Q.electron_gas}[name]()
    sysh = Q.System(ctx, spec)
    W = 256
    step, tau = (1.0, 0.05) if name == "heg" else (0.3, 0.02)
    wk = Q.Walkers(sysh, W, L.QMC_FP32_REFINE)
    wk.init(seed=61)
    wk.refresh()
    pos0 = wk.get_positions()                      # float values
    acc = wk.sweep(move, 1, 4, seed=909, step=step, tau=tau, max_drift=1.0)
    got = wk.get_positions()
    want, acc_o, _, mg = oracle.sweeps(spec, pos0, 1, 4, move, 909, step=step, tau=tau, max_drift=1.0,
                                       want_energy=False, want_margin=True)
    tol, band = (2e-5, 1e-3) if move == L.QMC_MOVE_ONE_GAUSS else (2e-4, 1e-2)
    same = np.all(np.abs(got - want) < tol, axis=(1, 2))
    unexplained = ~same & (mg > band)
    if move == L.QMC_MOVE_ONE_GAUSS:
        assert not unexplained.any(), (np.where(unexplained)[0], mg[unexplained])
    else:
        # near a node of the determinant grad D / D is a difference of nearly
        # equal FP32 terms, so a drift-diffusion proposal there can land
        # elsewhere than the FP64 one: at most 2 % of the walkers may do so
        assert unexplained.mean() <= 0.02, (np.where(unexplained)[0], mg[unexplained])
    assert same.mean() > 0.9, same.mean()
    assert acc > 0

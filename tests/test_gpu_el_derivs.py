"""dE_L/dp on the device (qmc_logderiv_batch's dEL output): the derivatives
of EnergyCalculator::local_energy (src/systems/methane.rs:1154-1182) in every
optimisable parameter, next to the SR log-derivatives of
src/systems/methane.rs:1186-1220 and src/systems/benzene.rs:726-756.

Tolerances: against the oracle's analytic form 1e-9 relative (both FP64);
against Richardson-extrapolated central differences of the device's own E_L
(steps 2h and h, h = 1e-4, through qmc_system_set_params) 1e-5 relative."""
import numpy as np
import pytest

import rust_qmc_gb300 as Q
from rust_qmc_gb300 import _lib as L
from tests.helpers import random_configs

pytestmark = pytest.mark.gpu

DISTINCT = [1.3, 1.7, 0.45, 0.3, 1.9, 2.4, 0.8, 1.1]


def spec_of(name):
    spec = {"ch4_min": Q.methane_minimal, "ch4_gto": Q.methane_gto, "c6h6": Q.benzene_minimal}[name]()
    p = np.asarray(spec.params(), dtype=np.float64)
    p[:8] = DISTINCT
    if len(p) > 8:
        p[8:] = [0.1, -0.2, 0.05, 0.3][: len(p) - 8]
    return spec.with_params(p)


def rel(a, b):
    return np.max(np.abs(a - b) / np.maximum(1.0, np.abs(b)))


@pytest.mark.parametrize("name", ["ch4_min", "ch4_gto", "c6h6"])
def test_el_derivatives_match_oracle(ctx, oracle, name):
    spec = spec_of(name)
    sysh = Q.System(ctx, spec)
    cfg = random_configs(spec, 48 if name == "c6h6" else 300, seed=17)
    O, E, dE, S, f, em = sysh.logderiv_batch(cfg, sums=True, el_derivs=True)
    assert dE.shape == (len(cfg), spec.n_params)
    want = oracle.el_derivatives(spec, cfg)
    assert rel(dE, want) < 1e-9, rel(dE, want)
    assert rel(O, oracle.log_derivatives(spec, cfg)) < 1e-10
    assert rel(E, oracle.evaluate(spec, cfg)["e_local"]) < 1e-9


@pytest.mark.parametrize("name", ["ch4_min", "c6h6"])
def test_el_derivatives_match_device_finite_differences(ctx, name):
    spec = spec_of(name)
    sysh = Q.System(ctx, spec)
    cfg = random_configs(spec, 16, seed=23)
    _, _, dE = sysh.logderiv_batch(cfg, el_derivs=True)
    p0 = sysh.get_params()
    h = 1e-4

    def el_at(p):
        sysh.set_params(p)
        return sysh.eval_batch(cfg, L.QMC_FP64)["e_local"]

    fd = np.zeros_like(dE)
    for k in range(len(p0)):
        d = []
        for hh in (2 * h, h):
            pp, pm = p0.copy(), p0.copy()
            pp[k] += hh
            pm[k] -= hh
            d.append((el_at(pp) - el_at(pm)) / (2 * hh))
        fd[:, k] = (4 * d[1] - d[0]) / 3
    sysh.set_params(p0)
    scale = np.maximum(np.abs(fd), 1e-3 * np.abs(fd).max())
    assert np.max(np.abs(dE - fd) / scale) < 1e-5


def test_el_derivatives_trait_adapter(ctx, oracle):
    spec = spec_of("ch4_min")
    sysh = Q.System(ctx, spec)
    r = random_configs(spec, 1, seed=5)[0]
    np.testing.assert_allclose(sysh.local_energy_derivatives(r), oracle.el_derivatives(spec, r)[0], rtol=1e-9,
                               atol=1e-9)

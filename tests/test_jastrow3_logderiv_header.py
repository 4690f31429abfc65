"""The Jastrow3 parameter log-derivatives and local-energy derivatives of
csrc/qmc_jastrow3_logderiv.h, compiled unchanged for the host with g++,
against the oracle's (src/correlation/jastrow.rs:326-391 generalised per spin
class and species; dE_L/dp from the oracle's el_derivs).  The device kernel
k_jastrow3_logderiv runs the same functions per walker."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import rust_qmc_gb300 as Q
from tests.helpers import random_configs

HERE = os.path.dirname(os.path.abspath(__file__))
HEADER_DIR = os.path.join(HERE, "..", "rust_qmc_gb300", "csrc")

HARNESS = r"""
#include <cstdio>
#include <vector>
#include "qmc_jastrow3_logderiv.h"
int main() {
    int W, N, n_up, n_nuc;
    if (std::scanf("%d %d %d %d", &W, &N, &n_up, &n_nuc) != 4) return 1;
    std::vector<double> p(8), nuc(5 * n_nuc), pos(3 * N);
    for (double& v : p) std::scanf("%lf", &v);
    for (double& v : nuc) std::scanf("%lf", &v);
    std::vector<double> grad(3 * N);
    for (int w = 0; w < W; ++w) {
        for (double& v : pos) std::scanf("%lf", &v);
        for (double& v : grad) std::scanf("%lf", &v);
        auto at = [&](int i, int c) { return pos[3 * i + c]; };
        auto gr = [&](int i, int c) { return grad[3 * i + c]; };
        double O[8], dE[8];
        qmc::jastrow3_log_derivatives(N, n_up, n_nuc, nuc.data(), p.data(), at, O);
        qmc::jastrow3_el_derivatives(N, n_up, n_nuc, nuc.data(), p.data(), at, gr, dE);
        for (int k = 0; k < 8; ++k) std::printf("%.17g ", O[k]);
        for (int k = 0; k < 8; ++k) std::printf("%.17g ", dE[k]);
        std::printf("\n");
    }
    return 0;
}
"""


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("j3")
    src = d / "harness.cpp"
    src.write_text(HARNESS)
    exe = d / "harness"
    subprocess.run([gxx, "-O2", "-std=c++17", "-I", HEADER_DIR, str(src), "-o", str(exe)], check=True)
    return str(exe)


def run_header(exe, spec, cfg, grad):
    """(O, dE_L/dp Jastrow columns) of the header for configurations cfg with
    grad ln|psi| per electron grad (both in the caller's electron order)."""
    spins = np.asarray(spec.spins)
    order = np.concatenate([np.where(spins > 0)[0], np.where(spins <= 0)[0]])   # up first, as at the ABI
    n_up = int((spins > 0).sum())
    nuc = np.column_stack([spec.nuc_pos, spec.nuc_charge, spec.nuc_species]).ravel()
    lines = ["%d %d %d %d" % (len(cfg), spec.n_elec, n_up, spec.n_nuc),
             " ".join("%.17g" % v for v in np.asarray(spec.jas)[:8]),
             " ".join("%.17g" % v for v in nuc)]
    for r, g in zip(cfg, grad):
        lines.append(" ".join("%.17g" % v for v in r[order].ravel()))
        lines.append(" ".join("%.17g" % v for v in g[order].ravel()))
    out = subprocess.run([exe], input="\n".join(lines) + "\n", capture_output=True, text=True, check=True).stdout
    res = np.array([[float(x) for x in l.split()] for l in out.strip().splitlines()])
    return res[:, :8], res[:, 8:]


@pytest.mark.parametrize("builder", ["c6h6", "ch4_gto"])
def test_header_matches_oracle(oracle, harness, builder):
    spec = Q.benzene_minimal() if builder == "c6h6" else Q.methane_gto(2.0, 3.0)
    p = np.asarray(spec.params(), dtype=np.float64)
    p[:8] = [1.3, 1.7, 0.45, 0.3, 1.9, 2.4, 0.8, 1.1]     # every parameter distinct
    spec = spec.with_params(p)
    cfg = random_configs(spec, 6, seed=31)
    grad = oracle.evaluate(spec, cfg)["grad"]
    got, got_de = run_header(harness, spec, cfg, grad)
    want = oracle.log_derivatives(spec, cfg)[:, :8]
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-12 * np.abs(want).max())
    # Jastrow columns of dE_L/dp: the header's form against the oracle's
    want_de = oracle.el_derivatives(spec, cfg)[:, :8]
    np.testing.assert_allclose(got_de, want_de, rtol=1e-10, atol=1e-10 * np.abs(want_de).max())

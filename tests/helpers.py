"""Shared helpers for the tests (configuration generators, FD checks)."""
import numpy as np


def random_configs(spec, W, seed, sigma=None):
    """Seeded configurations near the initial centres of the system."""
    rng = np.random.default_rng(seed)
    centres = np.array([spec.nuc_pos[i] if i >= 0 else np.zeros(3) for i in spec.init_nuc])
    s = spec.init_sigma if sigma is None else sigma
    return centres[None] + s * rng.standard_normal((W, spec.n_elec, 3))


def fd_grad_lap(O, spec, r, h=1e-4):
    """Central differences of ln|psi| (grad) and of psi (Laplacian / psi),
    as MultiWfn::numerical_derivative / numerical_laplacian do
    (src/wavefunction/traits.rs:62-90), Richardson-extrapolated from steps
    2h and h so that configurations near a node still compare tightly."""
    g1, l1 = _fd(O, spec, r, 2 * h)
    g2, l2 = _fd(O, spec, r, h)
    return (4 * g2 - g1) / 3, (4 * l2 - l1) / 3


def _fd(O, spec, r, h):
    N = spec.n_elec
    base = O.evaluate(spec, r)["logabs"][0]
    shifts = []
    for i in range(N):
        for a in range(3):
            for s in (+1, -1):
                rr = r.copy()
                rr[i, a] += s * h
                shifts.append(rr)
    l = O.evaluate(spec, np.array(shifts))["logabs"].reshape(N, 3, 2)
    grad = (l[:, :, 0] - l[:, :, 1]) / (2 * h)
    lap = np.sum(np.exp(l[:, :, 0] - base) + np.exp(l[:, :, 1] - base) - 2.0, axis=1) / (h * h)
    return grad, lap

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


def autocorrelation_time(x):
    """Integrated autocorrelation time by the initial positive sequence
    (src/sampling/vmc.rs:141-163)."""
    x = np.asarray(x, dtype=np.float64)
    n = len(x)
    m = x.mean()
    v = ((x - m) ** 2).mean()
    if n == 0 or v == 0.0:
        return 1.0
    tau = 1.0
    for t in range(1, n // 2):
        a = ((x[:-t] - m) * (x[t:] - m)).sum() / ((n - t) * v)
        if a < 0:
            break
        tau += 2.0 * a
    return tau


def blocking_error(x):
    """Blocking error with blocks of ceil(2 tau_int) (src/sampling/vmc.rs:166-188);
    returns (error, number of blocks)."""
    x = np.asarray(x, dtype=np.float64)
    bs = max(1, int(np.ceil(2.0 * autocorrelation_time(x))))
    nb = len(x) // bs
    if nb < 2:
        return 0.0, nb
    m = x[: nb * bs].reshape(nb, bs).mean(axis=1)
    return float(m.std(ddof=1) / np.sqrt(nb)), nb

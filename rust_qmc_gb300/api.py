"""Python face of the C ABI, shaped like the reference's traits.

``System`` exposes the batched calls (``eval_batch``, ``logderiv_batch``,
``forces_batch``) and, for drop-in use one configuration at a time, the
reference trait methods with their value conventions:

  MultiWfn (src/wavefunction/traits.rs:48-91)
      evaluate(r) -> psi, derivative(r) -> grad_i psi, laplacian(r) -> lap_i psi
  EnergyCalculator (src/sampling/traits.rs:6-8)
      local_energy(r)
  OptimizableWfn (src/wavefunction/traits.rs:98-115)
      num_params(), get_params(), set_params(p), log_derivatives(r)
  ForceCalculator (src/sampling/traits.rs:20-56)
      num_nuclei(), get_nuclei(), get_charges(), set_nuclei(R),
      hellmann_feynman_force(r), wfn_nuclear_gradient(r)

``Walkers`` is the device-resident ensemble (the samplers' walker vectors).
"""
import ctypes as C
import weakref

import numpy as np

from . import _lib as L

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def _d(a):
    return None if a is None else a.ctypes.data_as(_dp)


def _i(a):
    return None if a is None else a.ctypes.data_as(_ip)


class Context:
    """One CUDA device + stream (qmc_init / qmc_destroy)."""

    def __init__(self, device=0):
        self.lib = L.load_library()
        self._children = weakref.WeakSet()
        h = C.c_void_p()
        L.check(self.lib.qmc_init(device, C.byref(h)), "qmc_init")
        self.h = h

    def close(self):
        """Destroys the context; systems and walkers made from it close first."""
        for ch in list(getattr(self, "_children", ())):
            ch.close()
        if getattr(self, "h", None):
            self.lib.qmc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def record(self, slot):
        L.check(self.lib.qmc_ctx_event_record(self.h, slot), "qmc_ctx_event_record")

    def elapsed_ms(self, a, b):
        ms = C.c_float()
        L.check(self.lib.qmc_ctx_event_elapsed(self.h, a, b, C.byref(ms)), "qmc_ctx_event_elapsed")
        return float(ms.value)

    def synchronize(self):
        L.check(self.lib.qmc_ctx_synchronize(self.h), "qmc_ctx_synchronize")

    def flush_l2(self):
        L.check(self.lib.qmc_ctx_flush_l2(self.h), "qmc_ctx_flush_l2")

    def measure_peaks(self):
        """(FP32, FP64) FMA TFLOP/s measured on this GPU."""
        a, b = C.c_double(), C.c_double()
        L.check(self.lib.qmc_ctx_measure_peaks(self.h, C.byref(a), C.byref(b)), "qmc_ctx_measure_peaks")
        return a.value, b.value

    def launch_count(self):
        n = C.c_longlong()
        L.check(self.lib.qmc_ctx_launch_count(self.h, C.byref(n)), "qmc_ctx_launch_count")
        return int(n.value)


class PinnedArray:
    """A numpy view of page-locked host memory (qmc_host_alloc)."""

    def __init__(self, lib, shape, dtype=np.float64):
        self.lib = lib
        n = int(np.prod(shape)) * np.dtype(dtype).itemsize
        p = C.c_void_p()
        L.check(lib.qmc_host_alloc(n, C.byref(p)), "qmc_host_alloc")
        self.ptr = p
        buf = (C.c_char * n).from_address(p.value)
        self.array = np.frombuffer(buf, dtype=dtype).reshape(shape)

    def free(self):
        if self.ptr:
            self.array = None
            self.lib.qmc_host_free(self.ptr)
            self.ptr = None


class System:
    """A system handle (qmc_system_create) built from a SystemSpec."""

    def __init__(self, ctx, spec):
        self.ctx, self.spec, self.lib = ctx, spec, ctx.lib
        self._children = weakref.WeakSet()
        self._desc = spec.desc()
        h = C.c_void_p()
        L.check(self.lib.qmc_system_create(ctx.h, C.byref(self._desc), C.byref(h)), "qmc_system_create")
        self.h = h
        self.N = spec.n_elec
        ctx._children.add(self)

    def close(self):
        """Destroys the system; walker sets made from it close first."""
        for ch in list(getattr(self, "_children", ())):
            ch.close()
        if getattr(self, "h", None):
            self.lib.qmc_system_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- batched ------------------------------------------------------------
    def _pos(self, pos):
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        if pos.ndim == 2:
            pos = pos[None]
        if pos.shape[1:] != (self.N, 3):
            raise ValueError("positions must be W x %d x 3" % self.N)
        return pos

    def eval_batch(self, pos, precision=L.QMC_FP64):
        pos = self._pos(pos)
        W = pos.shape[0]
        out = dict(logabs=np.zeros(W), sign=np.zeros(W, np.int32), grad=np.zeros((W, self.N, 3)),
                   lap=np.zeros((W, self.N)), e_local=np.zeros(W))
        L.check(self.lib.qmc_eval_batch(self.h, W, _d(pos), precision, _d(out["logabs"]), _i(out["sign"]),
                                        _d(out["grad"]), _d(out["lap"]), _d(out["e_local"])), "qmc_eval_batch")
        return out

    def logderiv_batch(self, pos, sums=False, el_derivs=False):
        """(O, E_L[, dE_L/dp][, S, f, <E>]) per qmc_logderiv_batch: O [W, P] the
        log-derivatives, dE_L/dp [W, P] with el_derivs, the SR sums with sums."""
        pos = self._pos(pos)
        W, P = pos.shape[0], self.num_params()
        O, E = np.zeros((W, P)), np.zeros(W)
        dE = np.zeros((W, P)) if el_derivs else None
        S = np.zeros((P, P)) if sums else None
        f = np.zeros(P) if sums else None
        em = C.c_double()
        L.check(self.lib.qmc_logderiv_batch(self.h, W, _d(pos), _d(O), _d(E), _d(dE), _d(S), _d(f),
                                            C.byref(em) if sums else None), "qmc_logderiv_batch")
        out = (O, E) + ((dE,) if el_derivs else ())
        if sums:
            out += (S, f, em.value)
        return out

    def local_energy_derivatives(self, r):
        """d E_L / dp of one configuration (the E_L derivatives behind the SR
        and force interfaces)."""
        return self.logderiv_batch(r, el_derivs=True)[2][0]

    def ratio_batch(self, pos, e, r_new):
        """psi(moved)/psi for electron e moved to r_new[w] in each configuration,
        and grad_e ln psi at the moved configuration (qmc_ratio_batch)."""
        pos = self._pos(pos)
        W = pos.shape[0]
        r_new = np.ascontiguousarray(r_new, dtype=np.float64).reshape(W, 3)
        ratio, grad = np.zeros(W), np.zeros((W, 3))
        L.check(self.lib.qmc_ratio_batch(self.h, W, _d(pos), int(e), _d(r_new), _d(ratio), _d(grad)),
                "qmc_ratio_batch")
        return ratio, grad

    def forces_batch(self, pos, omega=True):
        """(F_hf, omega) per configuration; omega=False skips the wave
        function's nuclear gradient (and returns None for it), which benzene
        does not have (its ForceCalculator has the Hellmann-Feynman force only)."""
        pos = self._pos(pos)
        W = pos.shape[0]
        F = np.zeros((W, self.spec.n_nuc, 3))
        Om = np.zeros((W, self.spec.n_nuc, 3)) if omega else None
        L.check(self.lib.qmc_forces_batch(self.h, W, _d(pos), _d(F), _d(Om)), "qmc_forces_batch")
        return F, Om

    # -- OptimizableWfn -------------------------------------------------------
    def num_params(self):
        P = C.c_int()
        L.check(self.lib.qmc_system_num_params(self.h, C.byref(P)), "qmc_system_num_params")
        return P.value

    def get_params(self):
        p = np.zeros(self.num_params())
        L.check(self.lib.qmc_system_get_params(self.h, _d(p), len(p)), "qmc_system_get_params")
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float64)
        L.check(self.lib.qmc_system_set_params(self.h, _d(p), len(p)), "qmc_system_set_params")
        self.spec = self.spec.with_params(p)

    def log_derivatives(self, r):
        return self.logderiv_batch(r)[0][0]

    # -- MultiWfn / EnergyCalculator (single configuration) -------------------
    def evaluate(self, r):
        o = self.eval_batch(r)
        return float(o["sign"][0] * np.exp(o["logabs"][0]))

    def derivative(self, r):
        o = self.eval_batch(r)
        return o["grad"][0] * (o["sign"][0] * np.exp(o["logabs"][0]))

    def laplacian(self, r):
        o = self.eval_batch(r)
        return o["lap"][0] * (o["sign"][0] * np.exp(o["logabs"][0]))

    def local_energy(self, r):
        return float(self.eval_batch(r)["e_local"][0])

    # -- ForceCalculator -------------------------------------------------------
    def num_nuclei(self):
        return self.spec.n_nuc

    def get_nuclei(self):
        return self.spec.nuc_pos.copy()

    def get_charges(self):
        return self.spec.nuc_charge.copy()

    def set_nuclei(self, R):
        R = np.ascontiguousarray(R, dtype=np.float64).reshape(-1)
        L.check(self.lib.qmc_system_set_nuclei(self.h, _d(R), len(R) // 3), "qmc_system_set_nuclei")
        self.spec = self.spec.with_nuclei(R)

    def hellmann_feynman_force(self, r):
        return self.forces_batch(r)[0][0]

    def wfn_nuclear_gradient(self, r):
        return self.forces_batch(r)[1][0]


class Walkers:
    """Device-resident walker ensemble (qmc_walkers_*)."""

    def __init__(self, system, W, precision=L.QMC_FP64, capacity=None):
        self.sys, self.lib, self.W, self.precision = system, system.lib, W, precision
        h = C.c_void_p()
        if capacity is None:
            L.check(self.lib.qmc_walkers_create(system.h, W, precision, C.byref(h)), "qmc_walkers_create")
        else:
            L.check(self.lib.qmc_walkers_create_dmc(system.h, W, capacity, precision, C.byref(h)),
                    "qmc_walkers_create_dmc")
        self.h = h
        system._children.add(self)

    def close(self):
        if getattr(self, "h", None):
            self.lib.qmc_walkers_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def init(self, seed):
        L.check(self.lib.qmc_walkers_init(self.h, seed), "qmc_walkers_init")

    def set_positions(self, pos):
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        L.check(self.lib.qmc_walkers_set_positions(self.h, _d(pos)), "qmc_walkers_set_positions")

    def set_positions_ptr(self, ptr):
        L.check(self.lib.qmc_walkers_set_positions(self.h, C.cast(ptr, _dp)), "qmc_walkers_set_positions")

    def get_positions(self):
        pos = np.zeros((self.W, self.sys.N, 3))
        L.check(self.lib.qmc_walkers_get_positions(self.h, _d(pos)), "qmc_walkers_get_positions")
        return pos

    def refresh(self, want_energies=False):
        el = np.zeros(self.W) if want_energies else None
        s = C.c_double()
        L.check(self.lib.qmc_walkers_refresh(self.h, _d(el), C.byref(s)), "qmc_walkers_refresh")
        return (s.value, el) if want_energies else s.value

    def refresh_async(self):
        L.check(self.lib.qmc_walkers_refresh(self.h, None, None), "qmc_walkers_refresh")

    def rebuild_inverse(self):
        """Inverse Slater matrices, sign and log|psi| from the current
        positions, without E_L (asynchronous on the context stream)."""
        L.check(self.lib.qmc_walkers_rebuild_inverse(self.h), "qmc_walkers_rebuild_inverse")

    def sweep(self, move_kind, n_sweeps, step0, seed, step=0.3, tau=0.01, max_drift=1.0, count=True):
        acc = C.c_longlong()
        L.check(self.lib.qmc_walkers_sweep(self.h, move_kind, n_sweeps, step0, step, tau, max_drift, seed,
                                           C.byref(acc) if count else None), "qmc_walkers_sweep")
        return acc.value if count else None

    def state(self):
        la, sg, el = np.zeros(self.W), np.zeros(self.W, np.int32), np.zeros(self.W)
        L.check(self.lib.qmc_walkers_get_state(self.h, _d(la), _i(sg), _d(el)), "qmc_walkers_get_state")
        return la, sg, el

    def count(self):
        n = C.c_int()
        L.check(self.lib.qmc_walkers_count(self.h, C.byref(n)), "qmc_walkers_count")
        self.W = n.value
        return n.value

    def dmc_step(self, tau, e_ref, seed, step, max_drift=1.0, fixed_node=True, fp64_measure=False,
                 reference_diffusion=False, branch_cut=0.0):
        """One IS-DMC step; returns (new population, mean E_L of it).
        branch_cut > 0 clamps the branching energy to e_ref +- branch_cut."""
        n, em = C.c_int(), C.c_double()
        tau_move = tau if reference_diffusion else 0.5 * tau
        L.check(self.lib.qmc_walkers_dmc_step(self.h, tau, tau_move, max_drift, int(bool(fixed_node)), e_ref, seed, step,
                                              int(bool(fp64_measure)), float(branch_cut), C.byref(n), C.byref(em)),
                "qmc_walkers_dmc_step")
        self.W = n.value
        return n.value, em.value

    def status(self):
        f = C.c_int()
        L.check(self.lib.qmc_walkers_status(self.h, C.byref(f)), "qmc_walkers_status")
        return f.value


class Batch:
    """Walker sets of one context advanced together (qmc_batch_*): one sweep
    and one refresh per shape class, one CUDA graph per step."""

    def __init__(self, ctx, walkers):
        self.ctx, self.lib, self.walkers = ctx, ctx.lib, list(walkers)
        arr = (C.c_void_p * len(self.walkers))(*[w.h.value for w in self.walkers])
        h = C.c_void_p()
        L.check(self.lib.qmc_batch_create(ctx.h, len(self.walkers), arr, C.byref(h)), "qmc_batch_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.qmc_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def system_seed(self, seed, i):
        return int(self.lib.qmc_batch_system_seed(seed, i))

    def sweep(self, move_kind, n_sweeps, step0, seed, step=0.3, tau=0.01, max_drift=1.0):
        L.check(self.lib.qmc_batch_sweep(self.h, move_kind, n_sweeps, step0, step, tau, max_drift, seed),
                "qmc_batch_sweep")

    def refresh(self):
        e = np.zeros(len(self.walkers))
        L.check(self.lib.qmc_batch_refresh(self.h, _d(e)), "qmc_batch_refresh")
        return e

    def run_steps(self, move_kind, n_steps, sweeps_per_step, step0, seed, step=0.3, tau=0.01, max_drift=1.0):
        e = np.zeros((n_steps, len(self.walkers)))
        L.check(self.lib.qmc_batch_run_steps(self.h, move_kind, n_steps, sweeps_per_step, step0, step, tau,
                                             max_drift, seed, _d(e)), "qmc_batch_run_steps")
        return e


def roofline_model(spec, precision=L.QMC_FP32_REFINE, acceptance=0.5):
    """Algorithmic counts of the walker kernels for a system (qmc_roofline_model,
    host only): sweep operations per proposal, sweep state bytes per walker and
    launch, refresh operations and HBM bytes per walker."""
    desc = spec.desc()
    out = L.RooflineCounts()
    L.check(L.load_library().qmc_roofline_model(C.byref(desc), precision, acceptance, C.byref(out)),
            "qmc_roofline_model")
    return dict(sweep_flops_per_move=out.sweep_flops_per_move, sweep_state_bytes=out.sweep_state_bytes,
                refresh_flops=out.refresh_flops, refresh_bytes=out.refresh_bytes)


def batch_system_seed(seed, i):
    return int(L.load_library().qmc_batch_system_seed(seed, i))


def batch_run(ctx, systems, walkers_per_system, *, n_steps, n_burnin=0, move_kind=L.QMC_MOVE_ONE_GAUSS, step=0.3,
              tau=0.01, max_drift=1.0, precision=L.QMC_FP32_REFINE, refresh_every=64, seed=1):
    """VMC of many systems in one batch (qmc_batch_run); one result dict per system."""
    n = len(systems)
    p = L.RunParams()
    p.n_walkers, p.n_steps, p.n_burnin, p.move_kind = 0, n_steps, n_burnin, move_kind
    p.step, p.tau, p.max_drift, p.precision, p.refresh_every = step, tau, max_drift, precision, refresh_every
    res = (L.RunResult * n)()
    W = np.ascontiguousarray(walkers_per_system, dtype=np.int32)
    every = refresh_every if refresh_every > 0 else 1
    rows = (n_steps + every - 1) // every
    energies = np.zeros((rows, n))
    hs = (C.c_void_p * n)(*[s.h.value for s in systems])
    L.check(ctx.lib.qmc_batch_run(ctx.h, n, hs, _i(W), C.byref(p), seed, res, _d(energies)), "qmc_batch_run")
    out = []
    for i in range(n):
        r = res[i]
        out.append(dict(energy=r.energy, error=r.error, autocorrelation_time=r.autocorrelation_time,
                        acceptance_rate=r.acceptance_rate, variance=r.variance, n_samples=r.n_samples,
                        status_flags=r.status_flags, energies=energies[:, i].copy()))
    return out


def vmc_run(system, *, n_walkers, n_steps, n_burnin=0, move_kind=L.QMC_MOVE_ALL_BOX, step=1.0, tau=0.01,
            max_drift=1.0, precision=L.QMC_FP64, refresh_every=64, seed=1, target_acceptance=0.0,
            adaptation_interval=100, min_step=0.0, max_step=0.0):
    """MCMCSimulation::run / DriftDiffusionVMC::run on the device; with
    target_acceptance > 0 the step (or tau) adapts every adaptation_interval
    steps as the reference's samplers do (src/sampling/vmc.rs:122-128,
    397-402)."""
    p = L.RunParams()
    p.n_walkers, p.n_steps, p.n_burnin, p.move_kind = n_walkers, n_steps, n_burnin, move_kind
    p.step, p.tau, p.max_drift, p.precision, p.refresh_every = step, tau, max_drift, precision, refresh_every
    p.target_acceptance, p.adaptation_interval = target_acceptance, adaptation_interval
    p.min_step, p.max_step = min_step, max_step
    res = L.RunResult()
    energies = np.zeros(n_steps)
    L.check(system.lib.qmc_vmc_run(system.h, C.byref(p), seed, C.byref(res), _d(energies)), "qmc_vmc_run")
    return dict(energy=res.energy, error=res.error, autocorrelation_time=res.autocorrelation_time,
                acceptance_rate=res.acceptance_rate, variance=res.variance, n_samples=res.n_samples,
                status_flags=res.status_flags, energies=energies[:res.n_samples], final_step=res.final_step)


def _dmc_params(n_walkers, n_steps, n_burnin, tau, max_drift, precision, refresh_every, e_ref_damping, fixed_node,
                reference_diffusion, branch_cut=0.0):
    p = L.RunParams()
    p.n_walkers, p.n_steps, p.n_burnin, p.move_kind = n_walkers, n_steps, n_burnin, L.QMC_MOVE_ONE_DRIFT
    p.tau, p.max_drift, p.precision, p.refresh_every = tau, max_drift, precision, refresh_every
    p.e_ref_damping, p.fixed_node = e_ref_damping, int(bool(fixed_node))
    p.reference_diffusion = int(bool(reference_diffusion))
    p.branch_cut = float(branch_cut)
    return p


def _run_dict(res, energies):
    return dict(energy=res.energy, error=res.error, autocorrelation_time=res.autocorrelation_time,
                acceptance_rate=res.acceptance_rate, variance=res.variance, n_samples=res.n_samples,
                status_flags=res.status_flags, avg_population=res.avg_population,
                energies=energies[:res.n_samples])


def dmc_run(system, *, n_walkers, n_steps, n_burnin=0, tau=0.005, max_drift=1.0, precision=L.QMC_FP64,
            refresh_every=1, e_ref_damping=0.5, fixed_node=True, reference_diffusion=False, seed=1, branch_cut=0.0):
    """ImportanceSampledDMC::run (energy part) on the device; branch_cut > 0
    clamps the branching energy to E_ref +- branch_cut (0: the reference's
    branching)."""
    p = _dmc_params(n_walkers, n_steps, n_burnin, tau, max_drift, precision, refresh_every, e_ref_damping,
                    fixed_node, reference_diffusion, branch_cut)
    res = L.RunResult()
    energies = np.zeros(n_steps)
    L.check(system.lib.qmc_dmc_run(system.h, C.byref(p), seed, C.byref(res), _d(energies)), "qmc_dmc_run")
    return _run_dict(res, energies)


def dmc_run_forces(system, *, n_walkers, n_steps, n_burnin=0, tau=0.005, max_drift=1.0, precision=L.QMC_FP64,
                   refresh_every=1, e_ref_damping=0.5, fixed_node=True, reference_diffusion=False,
                   n_vmc_equilibrate=500, n_vmc_force_samples=2000, seed=1):
    """ImportanceSampledDMC::run with the mixed, VMC and extrapolated
    Hellmann-Feynman force estimators (qmc_dmc_run_forces); the energy part is
    dmc_run's with the same arguments."""
    p = _dmc_params(n_walkers, n_steps, n_burnin, tau, max_drift, precision, refresh_every, e_ref_damping,
                    fixed_node, reference_diffusion)
    res = L.RunResult()
    energies = np.zeros(n_steps)
    n = system.num_nuclei()
    fm, fv, fe = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 3))
    L.check(system.lib.qmc_dmc_run_forces(system.h, C.byref(p), n_vmc_equilibrate, n_vmc_force_samples, seed,
                                          C.byref(res), _d(energies), _d(fm), _d(fv), _d(fe)),
            "qmc_dmc_run_forces")
    out = _run_dict(res, energies)
    out.update(forces_mixed=fm, forces_vmc=fv, forces_extrapolated=fe)
    return out

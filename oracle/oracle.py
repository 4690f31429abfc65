"""ctypes wrapper of oracle/build/libqmc_oracle.so (test infrastructure).

Takes the product's SystemSpec objects only as plain data (the descriptor
layout is shared with include/qmc.h; tests check the sizes agree).
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_u32p = C.POINTER(C.c_uint32)
_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        l = C.CDLL(path)
        vp = C.c_void_p
        l.orc_desc_size.restype = C.c_int
        l.orc_philox.argtypes = [_u32p, _u32p, _u32p]
        l.orc_eval.argtypes = [vp, C.c_int, _dp, _dp, _ip, _dp, _dp, _dp, C.c_int]
        l.orc_jastrow.argtypes = [vp, _dp, _dp, _dp, _dp]
        l.orc_logderiv.argtypes = [vp, C.c_int, _dp, _dp, C.c_int]
        l.orc_el_derivs.argtypes = [vp, C.c_int, _dp, _dp, C.c_int]
        l.orc_forces.argtypes = [vp, C.c_int, _dp, _dp, _dp, C.c_int]
        l.orc_forces_fd.argtypes = [vp, C.c_int, _dp, C.c_double, _dp]
        l.orc_init.argtypes = [vp, C.c_int, C.c_uint32, C.c_uint64, _dp]
        l.orc_sweeps.argtypes = [vp, C.c_int, C.c_uint32, _dp, C.c_int, C.c_uint64, C.c_int, C.c_double,
                                 C.c_double, C.c_double, C.c_uint64, _ip, _dp, _dp, C.c_int]
        l.orc_dmc.argtypes = [vp, C.c_int, _dp, C.c_int, C.c_uint64, C.c_double, C.c_double, C.c_double, C.c_int,
                              C.c_double, C.c_double,
                              C.c_int, C.c_uint64, C.c_int, _dp, _ip, _ip, _dp, _dp, C.c_int]
        l.orc_dmc.restype = C.c_int
        l.orc_heg_ewald.argtypes = [vp, _dp, C.c_double, C.c_int]
        l.orc_heg_ewald.restype = C.c_double
        _lib = l
    return _lib


def _d(a):
    return None if a is None else a.ctypes.data_as(_dp)


def _i(a):
    return None if a is None else a.ctypes.data_as(_ip)


def threads_default():
    return os.cpu_count() or 1


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().orc_philox(c, k, o)
    return tuple(int(x) for x in o)


def evaluate(spec, pos, threads=None):
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    if pos.ndim == 2:
        pos = pos[None]
    W, N = pos.shape[0], spec.n_elec
    d = spec.desc()
    out = dict(logabs=np.zeros(W), sign=np.zeros(W, np.int32), grad=np.zeros((W, N, 3)), lap=np.zeros((W, N)),
               e_local=np.zeros(W))
    lib().orc_eval(C.byref(d), W, _d(pos), _d(out["logabs"]), _i(out["sign"]), _d(out["grad"]), _d(out["lap"]),
                   _d(out["e_local"]), threads or threads_default())
    return out


def jastrow(spec, r):
    r = np.ascontiguousarray(r, dtype=np.float64)
    d = spec.desc()
    J = C.c_double()
    g = np.zeros((spec.n_elec, 3))
    l = np.zeros(spec.n_elec)
    lib().orc_jastrow(C.byref(d), _d(r), C.byref(J), _d(g), _d(l))
    return J.value, g, l


def log_derivatives(spec, pos, threads=None):
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    if pos.ndim == 2:
        pos = pos[None]
    W = pos.shape[0]
    O = np.zeros((W, spec.n_params))
    d = spec.desc()
    lib().orc_logderiv(C.byref(d), W, _d(pos), _d(O), threads or threads_default())
    return O


def el_derivatives(spec, pos, threads=None):
    """dE_L / dp per configuration [W, P] (analytic, oracle's el_derivs)."""
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    if pos.ndim == 2:
        pos = pos[None]
    W = pos.shape[0]
    dE = np.zeros((W, spec.n_params))
    d = spec.desc()
    lib().orc_el_derivs(C.byref(d), W, _d(pos), _d(dE), threads or threads_default())
    return dE


def el_derivatives_fd(spec, pos, h=1e-4, threads=None):
    """Central finite differences of the oracle's E_L in each parameter."""
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    if pos.ndim == 2:
        pos = pos[None]
    p0 = np.asarray(spec.params(), dtype=np.float64)
    out = np.zeros((pos.shape[0], len(p0)))
    for k in range(len(p0)):
        pp, pm = p0.copy(), p0.copy()
        pp[k] += h
        pm[k] -= h
        ep = evaluate(spec.with_params(pp), pos, threads)["e_local"]
        em = evaluate(spec.with_params(pm), pos, threads)["e_local"]
        out[:, k] = (ep - em) / (2 * h)
    return out


def forces(spec, pos, threads=None):
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    if pos.ndim == 2:
        pos = pos[None]
    W = pos.shape[0]
    F = np.zeros((W, spec.n_nuc, 3))
    Om = np.zeros((W, spec.n_nuc, 3))
    d = spec.desc()
    lib().orc_forces(C.byref(d), W, _d(pos), _d(F), _d(Om), threads or threads_default())
    return F, Om


def nuclear_gradient_fd(spec, pos, h=1e-5):
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    if pos.ndim == 2:
        pos = pos[None]
    W = pos.shape[0]
    Om = np.zeros((W, spec.n_nuc, 3))
    d = spec.desc()
    lib().orc_forces_fd(C.byref(d), W, _d(pos), h, _d(Om))
    return Om


def init_positions(spec, W, seed, walker0=0):
    pos = np.zeros((W, spec.n_elec, 3))
    d = spec.desc()
    lib().orc_init(C.byref(d), W, walker0, seed, _d(pos))
    return pos


def sweeps(spec, pos, n_sweeps, sweep0, move_kind, seed, step=0.3, tau=0.01, max_drift=1.0, walker0=0,
           threads=None, want_energy=True, want_margin=False):
    """Reference-algorithm Monte Carlo sweeps; returns (pos, accepted, e_local),
    plus with want_margin the per-walker smallest relative distance between
    an acceptance uniform and its acceptance probability."""
    pos = np.array(pos, dtype=np.float64, copy=True)
    W = pos.shape[0]
    acc = np.zeros(W, np.int32)
    el = np.zeros(W) if want_energy else None
    mg = np.zeros(W) if want_margin else None
    d = spec.desc()
    lib().orc_sweeps(C.byref(d), W, walker0, _d(pos), n_sweeps, sweep0, move_kind, step, tau, max_drift, seed,
                     _i(acc), _d(el), _d(mg), threads or threads_default())
    if want_margin:
        return pos, acc, el, mg
    return pos, acc, el


def dmc(spec, pos, n_steps, tau, e_ref, target, seed, step0=0, max_drift=1.0, fixed_node=True, kappa=0.5,
        cap=None, threads=None, reference_diffusion=False, branch_cut=0.0):
    """Reference-algorithm IS-DMC with the shared random stream.
    Returns (final positions, per-step populations, per-step mean E_L, E_ref)."""
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    W0 = pos.shape[0]
    cap = cap or 4 * target
    out = np.zeros((cap, spec.n_elec, 3))
    Wout = C.c_int()
    pops = np.zeros(n_steps, np.int32)
    en = np.zeros(n_steps)
    er = C.c_double(e_ref)
    d = spec.desc()
    tau_move = tau if reference_diffusion else 0.5 * tau
    done = lib().orc_dmc(C.byref(d), W0, _d(pos), n_steps, step0, tau, tau_move, max_drift, int(bool(fixed_node)),
                         kappa, float(branch_cut), target,
                         seed, cap, _d(out), C.byref(Wout), _i(pops), _d(en), C.byref(er), threads or threads_default())
    return out[:Wout.value], pops[:done], en[:done], er.value


def heg_ewald(spec, r, alphaL=0.0, kmax=0):
    r = np.ascontiguousarray(r, dtype=np.float64)
    d = spec.desc()
    return lib().orc_heg_ewald(C.byref(d), _d(r), alphaL, kmax)

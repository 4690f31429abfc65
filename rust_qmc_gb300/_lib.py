"""ctypes binding of libqmc_gb300.so (the C ABI declared in include/qmc.h).

The shared library is built in-tree by ``rust_qmc_gb300.build.build()``.  There
is no fallback implementation: if the library cannot be loaded every entry
point raises ``QMCError``.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libqmc_gb300.so")

QMC_OK, QMC_ERR_ARG, QMC_ERR_CUDA, QMC_ERR_TIMEOUT, QMC_ERR_SINGULAR = 0, 1, 2, 3, 4
QMC_ERR_POPULATION, QMC_ERR_NONFINITE, QMC_ERR_UNSUPPORTED, QMC_ERR_NOMEM = 5, 6, 7, 8
QMC_FP64, QMC_FP32_REFINE = 0, 1
QMC_BASIS_GTO, QMC_BASIS_STO, QMC_BASIS_PW = 0, 1, 2
QMC_JAS_NONE, QMC_JAS_PADE_F, QMC_JAS_PADE_EEN, QMC_JAS_HEG = 0, 1, 2, 3
QMC_MOVE_ALL_GAUSS, QMC_MOVE_ALL_BOX, QMC_MOVE_ONE_GAUSS, QMC_MOVE_ONE_DRIFT = 0, 1, 2, 3
QMC_QUIRK_J2_GRAD, QMC_QUIRK_J2_LAP, QMC_QUIRK_HEG_EWALD, QMC_QUIRK_HEG_CROSS = 1, 2, 4, 8

_ip = C.POINTER(C.c_int)
_dp = C.POINTER(C.c_double)


class SystemDesc(C.Structure):
    """Mirror of ``qmc_system_desc``."""
    _fields_ = [
        ("n_elec", C.c_int), ("spins", _ip),
        ("n_nuc", C.c_int), ("nuc_pos", _dp), ("nuc_charge", _dp), ("nuc_species", _ip),
        ("basis_kind", C.c_int), ("n_ao", C.c_int),
        ("ao_nuc", _ip), ("ao_l", _ip), ("ao_m", _ip), ("ao_prim_off", _ip),
        ("prim_exp", _dp), ("prim_coef", _dp), ("prim_pow", _ip),
        ("n_mo", C.c_int), ("mo_coef", _dp), ("occ", _ip),
        ("jastrow_kind", C.c_int), ("jas_F", C.c_double), ("jas", C.c_double * 8),
        ("n_rot", C.c_int), ("rot_occ", _ip), ("rot_virt", _ip), ("rot_angle", _dp),
        ("quirks", C.c_int), ("init_nuc", _ip), ("init_sigma", C.c_double),
        ("box_L", C.c_double), ("reserved", C.c_int * 4),
    ]


class RunParams(C.Structure):
    """Mirror of ``qmc_run_params``."""
    _fields_ = [
        ("n_walkers", C.c_int), ("n_steps", C.c_int), ("n_burnin", C.c_int), ("move_kind", C.c_int),
        ("step", C.c_double), ("tau", C.c_double), ("max_drift", C.c_double),
        ("precision", C.c_int), ("refresh_every", C.c_int), ("e_ref_damping", C.c_double),
        ("fixed_node", C.c_int), ("reference_diffusion", C.c_int),
        ("target_acceptance", C.c_double), ("adaptation_interval", C.c_int), ("min_step", C.c_double),
        ("max_step", C.c_double), ("branch_cut", C.c_double), ("reserved", C.c_int * 2),
    ]


class RooflineCounts(C.Structure):
    """Mirror of ``qmc_roofline_counts``."""
    _fields_ = [
        ("sweep_flops_per_move", C.c_double), ("sweep_state_bytes", C.c_double),
        ("refresh_flops", C.c_double), ("refresh_bytes", C.c_double), ("reserved", C.c_double * 4),
    ]


class RunResult(C.Structure):
    """Mirror of ``qmc_run_result``."""
    _fields_ = [
        ("energy", C.c_double), ("error", C.c_double), ("autocorrelation_time", C.c_double),
        ("acceptance_rate", C.c_double), ("variance", C.c_double), ("n_samples", C.c_int),
        ("status_flags", C.c_int), ("avg_population", C.c_double), ("final_step", C.c_double),
        ("reserved", C.c_double * 3),
    ]


class QMCError(RuntimeError):
    def __init__(self, code, where=""):
        self.code = code
        msg = _status_string(code)
        super().__init__("%s failed: %s (status %d)" % (where, msg, code))


_vp = C.c_void_p
_u64 = C.c_uint64
# name -> argtypes (all functions return int unless listed in _RESTYPES)
PROTOTYPES = {
    "qmc_init": [C.c_int, C.POINTER(_vp)],
    "qmc_destroy": [_vp],
    "qmc_status_string": [C.c_int],
    "qmc_version": [],
    "qmc_system_create": [_vp, C.POINTER(SystemDesc), C.POINTER(_vp)],
    "qmc_system_destroy": [_vp],
    "qmc_system_check": [C.POINTER(SystemDesc), _ip],
    "qmc_system_num_params": [_vp, _ip],
    "qmc_system_get_params": [_vp, _dp, C.c_int],
    "qmc_system_set_params": [_vp, _dp, C.c_int],
    "qmc_system_set_nuclei": [_vp, _dp, C.c_int],
    "qmc_eval_batch": [_vp, C.c_int, _dp, C.c_int, _dp, _ip, _dp, _dp, _dp],
    "qmc_logderiv_batch": [_vp, C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _dp],
    "qmc_forces_batch": [_vp, C.c_int, _dp, _dp, _dp],
    "qmc_walkers_create": [_vp, C.c_int, C.c_int, C.POINTER(_vp)],
    "qmc_walkers_destroy": [_vp],
    "qmc_walkers_init": [_vp, _u64],
    "qmc_walkers_set_positions": [_vp, _dp],
    "qmc_walkers_get_positions": [_vp, _dp],
    "qmc_walkers_refresh": [_vp, _dp, _dp],
    "qmc_walkers_rebuild_inverse": [_vp],
    "qmc_walkers_sweep": [_vp, C.c_int, C.c_int, _u64, C.c_double, C.c_double, C.c_double, _u64,
                          C.POINTER(C.c_longlong)],
    "qmc_walkers_get_state": [_vp, _dp, _ip, _dp],
    "qmc_walkers_status": [_vp, _ip],
    "qmc_vmc_run": [_vp, C.POINTER(RunParams), _u64, C.POINTER(RunResult), _dp],
    "qmc_dmc_run": [_vp, C.POINTER(RunParams), _u64, C.POINTER(RunResult), _dp],
    "qmc_dmc_run_forces": [_vp, C.POINTER(RunParams), C.c_int, C.c_int, _u64, C.POINTER(RunResult), _dp, _dp, _dp,
                           _dp],
    "qmc_walkers_create_dmc": [_vp, C.c_int, C.c_int, C.c_int, C.POINTER(_vp)],
    "qmc_walkers_count": [_vp, _ip],
    "qmc_walkers_dmc_step": [_vp, C.c_double, C.c_double, C.c_double, C.c_int, C.c_double, _u64, _u64, C.c_int,
                             C.c_double, _ip, _dp],
    "qmc_ctx_event_record": [_vp, C.c_int],
    "qmc_ctx_event_elapsed": [_vp, C.c_int, C.c_int, C.POINTER(C.c_float)],
    "qmc_ctx_synchronize": [_vp],
    "qmc_ctx_flush_l2": [_vp],
    "qmc_ctx_launch_count": [_vp, C.POINTER(C.c_longlong)],
    "qmc_ctx_measure_peaks": [_vp, _dp, _dp],
    "qmc_host_alloc": [C.c_size_t, C.POINTER(_vp)],
    "qmc_host_free": [_vp],
    "qmc_sr_sums_noalloc": [_dp, _dp, C.c_int, C.c_int, _dp, _vp],
    "qmc_ratio_batch": [_vp, C.c_int, _dp, C.c_int, _dp, _dp, _dp],
    "qmc_roofline_model": [C.POINTER(SystemDesc), C.c_int, C.c_double, C.POINTER(RooflineCounts)],
    "qmc_batch_system_seed": [_u64, C.c_int],
    "qmc_batch_create": [_vp, C.c_int, C.POINTER(_vp), C.POINTER(_vp)],
    "qmc_batch_destroy": [_vp],
    "qmc_batch_sweep": [_vp, C.c_int, C.c_int, _u64, C.c_double, C.c_double, C.c_double, _u64],
    "qmc_batch_refresh": [_vp, _dp],
    "qmc_batch_run_steps": [_vp, C.c_int, C.c_int, C.c_int, _u64, C.c_double, C.c_double, C.c_double, _u64, _dp],
    "qmc_batch_run": [_vp, C.c_int, C.POINTER(_vp), _ip, C.POINTER(RunParams), _u64, C.POINTER(RunResult), _dp],
}
_RESTYPES = {"qmc_status_string": C.c_char_p, "qmc_batch_system_seed": _u64}

_lib = None
_load_error = None


def load_library(path=None):
    """Load (once) and return the CDLL; raises QMCError if it is unusable."""
    global _lib, _load_error
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        _load_error = "libqmc_gb300.so not built (run rust_qmc_gb300.build.build())"
        raise QMCError(QMC_ERR_CUDA, _load_error)
    lib = C.CDLL(p)
    for name, args in PROTOTYPES.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = _RESTYPES.get(name, C.c_int)
    _lib = lib
    return lib


def _status_string(code):
    try:
        return load_library().qmc_status_string(code).decode()
    except Exception:
        return "status %d" % code


def check(rc, where):
    if rc != QMC_OK:
        raise QMCError(rc, where)

"""CPU tests of the C ABI library: it builds, loads, exports every symbol
include/qmc.h declares, validates system descriptions on the host, and
reports the absence of a GPU as an error instead of falling back."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

import rust_qmc_gb300 as Q
from rust_qmc_gb300 import _lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    text = open(os.path.join(ROOT, "include", "qmc.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*|uint64_t)\s+(qmc_\w+)\s*\(", text, re.M)))


def test_header_declares_expected_surface():
    names = header_functions()
    for n in ["qmc_init", "qmc_system_create", "qmc_eval_batch", "qmc_logderiv_batch", "qmc_forces_batch",
              "qmc_walkers_sweep", "qmc_walkers_refresh", "qmc_vmc_run", "qmc_dmc_run", "qmc_batch_create",
              "qmc_batch_sweep", "qmc_batch_refresh", "qmc_batch_run_steps", "qmc_batch_run",
              "qmc_batch_system_seed"]:
        assert n in names


def test_library_exports_every_declared_symbol(qmc_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", L.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\s[TW]\s+(\w+)$", out, re.M))
    missing = [n for n in header_functions() if n not in exported]
    assert not missing, missing
    # and the ctypes prototypes cover the same set
    assert set(header_functions()) == set(L.PROTOTYPES), set(header_functions()) ^ set(L.PROTOTYPES)


def test_status_strings(qmc_lib):
    assert qmc_lib.qmc_version() >= 100
    for code in range(9):
        assert qmc_lib.qmc_status_string(code)
    assert b"unknown" in qmc_lib.qmc_status_string(99)


@pytest.mark.parametrize("builder,shape", [(lambda: Q.h2_mo(), 0), (lambda: Q.lithium_atom(), 1),
                                           (lambda: Q.methane_gto(), 2), (lambda: Q.methane_minimal(), 3),
                                           (lambda: Q.benzene_minimal(), 4), (lambda: Q.electron_gas(), 5),
                                           (lambda: Q.electron_gas(reference_quirks=True), 5)])
def test_system_check_maps_shapes(qmc_lib, builder, shape):
    spec = builder()
    d = spec.desc()
    got = C.c_int(-9)
    assert qmc_lib.qmc_system_check(C.byref(d), C.byref(got)) == L.QMC_OK
    assert got.value == shape


def test_system_check_rejects_bad_descriptions(qmc_lib):
    spec = Q.methane_minimal()
    bad = spec.copy()
    bad.spins = np.array([1] * 5 + [2] * 5, np.int32)
    assert qmc_lib.qmc_system_check(C.byref(bad.desc()), None) == L.QMC_ERR_ARG
    bad = spec.copy()
    bad.occ = np.array([0, 1, 2, 3, 99] * 2, np.int32)
    assert qmc_lib.qmc_system_check(C.byref(bad.desc()), None) == L.QMC_ERR_ARG
    bad = spec.copy()
    bad.ao_m = bad.ao_m.copy()
    bad.ao_m[3] = 0  # p triplet no longer complete
    assert qmc_lib.qmc_system_check(C.byref(bad.desc()), None) == L.QMC_ERR_ARG
    # an electron count with no compiled kernel is unsupported, not an error
    odd = Q.h2_mo()
    odd.spins = np.array([1, 1], np.int32)
    assert qmc_lib.qmc_system_check(C.byref(odd.desc()), None) == L.QMC_ERR_UNSUPPORTED
    assert qmc_lib.qmc_system_check(None, None) == L.QMC_ERR_ARG


def _gpu_visible():
    try:
        return subprocess.run(["nvidia-smi", "-L"], capture_output=True, timeout=20).returncode == 0
    except Exception:
        return False


@pytest.mark.skipif(_gpu_visible(), reason="a GPU is present; covered by the gpu tests")
def test_no_gpu_is_an_error_not_a_fallback(qmc_lib):
    h = C.c_void_p()
    assert qmc_lib.qmc_init(0, C.byref(h)) == L.QMC_ERR_CUDA
    assert not h.value
    with pytest.raises(Q.QMCError):
        Q.Context(0)


def test_batch_system_seed_is_splitmix64(qmc_lib):
    """Per-system Philox keys of a batch: SplitMix64 of seed + (i+1) x golden."""
    M = (1 << 64) - 1

    def splitmix(seed, i):
        z = (seed + 0x9E3779B97F4A7C15 * (i + 1)) & M
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
        return z ^ (z >> 31)

    for seed in (0, 1, 0x51A7E5, M):
        keys = [Q.batch_system_seed(seed, i) for i in range(64)]
        assert keys == [splitmix(seed, i) for i in range(64)]
        assert len(set(keys)) == 64


def test_roofline_model_counts(qmc_lib):
    """Host-only algorithmic counts (qmc_roofline_model) for the 9-AO CH4
    workload: 596 FP32 operations per proposal plus 105 per accepted move
    (Sherman-Morrison), 648 bytes of FP32 walker state read and written per
    sweep launch, and the two-pass refresh scratch in the refresh bytes."""
    spec = Q.methane_minimal()
    c = Q.roofline_model(spec, L.QMC_FP32_REFINE, 0.0)
    assert c["sweep_flops_per_move"] == pytest.approx(596.0)
    c = Q.roofline_model(spec, L.QMC_FP32_REFINE, 1.0)
    assert c["sweep_flops_per_move"] == pytest.approx(701.0)
    assert c["sweep_state_bytes"] == pytest.approx(2 * ((3 * 10 + 50) * 4 + 4))
    rows = 2 * 8 * 10 * (5 * 5 + 7)
    assert c["refresh_bytes"] == pytest.approx(3 * 10 * 4 + 50 * 4 + 20 + rows)
    c64 = Q.roofline_model(spec, L.QMC_FP64, 0.5)
    assert c64["sweep_state_bytes"] == pytest.approx(2 * ((3 * 10 + 50) * 8 + 4))
    assert c64["refresh_bytes"] == pytest.approx(3 * 10 * 8 + 50 * 8 + 20)
    for spec in (Q.h2_mo(), Q.lithium_atom(), Q.benzene_minimal(), Q.electron_gas()):
        c = Q.roofline_model(spec, L.QMC_FP32_REFINE, 0.5)
        assert all(v > 0 for v in c.values())
    with pytest.raises(Q.QMCError):
        Q.roofline_model(Q.methane_minimal(), L.QMC_FP32_REFINE, 1.5)

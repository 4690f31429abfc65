"""rust_qmc_gb300 -- GB300 (sm_103a) walker-ensemble Slater-Jastrow QMC.

A from-scratch GPU implementation of the walker path of rust_qmc (VMC
Metropolis and drift-diffusion sampling, local energies, parameter and
nuclear derivatives) behind the C ABI of include/qmc.h.  This package is the
ctypes face of that library plus the system builders; all numerical work
runs in libqmc_gb300.so.
"""
from . import _lib
from ._lib import QMCError, load_library
from .api import (Batch, Context, PinnedArray, System, Walkers, batch_run, batch_system_seed, dmc_run, dmc_run_forces,
                  roofline_model, vmc_run)
from .systems import (SystemSpec, h2_mo, lithium_atom, methane_gto, methane_minimal, benzene_minimal, benzene_gto, electron_gas,
                      heg_k_vectors, monkhorst_pack_grid, jastrow3_params,
                      reference_params_from_general, seeded_orthonormal, philox4x32, SEED_BASE)

__all__ = ["QMCError", "load_library", "Context", "PinnedArray", "System", "Walkers", "Batch", "batch_run",
           "batch_system_seed", "roofline_model", "vmc_run", "dmc_run", "dmc_run_forces", "SystemSpec",
           "h2_mo", "lithium_atom", "methane_gto", "methane_minimal", "benzene_minimal", "benzene_gto", "electron_gas", "heg_k_vectors", "monkhorst_pack_grid", "jastrow3_params",
           "reference_params_from_general", "seeded_orthonormal", "philox4x32", "SEED_BASE", "_lib"]

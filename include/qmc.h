/*
 * qmc.h -- C ABI of the GB300 walker-ensemble QMC library (libqmc_gb300.so).
 *
 * The library replaces the per-configuration Rust trait calls of rust_qmc's
 * Slater-Jastrow walker path with batched calls over W walkers resident in
 * GPU memory.  Every entry point below names the reference interface it
 * replaces (paths are relative to the rust_qmc source tree).
 *
 * Conventions
 *  - Plain C types only; no pointer is retained after a call returns.
 *  - Host buffers are owned by the caller; device state lives behind handles.
 *  - Every function returns a qmc_status (0 = success).  The library never
 *    aborts or traps; a CUDA error is reported as QMC_ERR_CUDA.
 *  - Positions are double precision, W x n_elec x 3, electrons in the
 *    caller's (reference) order.  Internally electrons are regrouped into
 *    contiguous spin sectors (spin +1 first, each sector in ascending caller
 *    index); per-electron outputs are returned in the caller's order.
 *  - psi is reported as (log|psi|, sign) instead of the reference's raw psi;
 *    gradients are grad_i psi / psi, Laplacians lap_i psi / psi.
 *  - One context = one CUDA stream; calls on one context are serialised.
 *  - Handles may be destroyed in any order.  Destroying a context that still
 *    has systems, or a system that still has walker sets, releases the handle
 *    at once (it accepts no further calls) and frees its memory when its last
 *    child is destroyed; the children stay fully usable until then.
 *
 * Random numbers: Philox4x32-10 keyed by the 64-bit seed, counter
 *   c0 = walker id, c1 = step (low 32 bits), c2 = electron / sub-index,
 *   c3 = tag | (step bits 32..47) << 16,  tag 1 proposal, 2 accept,
 *   3 initial position, 4 branching.
 * A single-electron move uses one call (tag 1, c2 = internal electron
 * index): the low 24 bits of words 0-3 are two Box-Muller pairs (three
 * displacement components used), the top bytes of words 0-2 the acceptance
 * uniform.  All-electron steps draw tag 1 per electron (32-bit uniforms) and
 * tag 2 once for acceptance.
 * Trajectories therefore depend only on (seed, walker id, step), never on the
 * launch geometry.
 */
#ifndef QMC_GB300_H
#define QMC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum {
    QMC_OK = 0,
    QMC_ERR_ARG = 1,          /* bad argument / size mismatch (reference: assert_eq! panics) */
    QMC_ERR_CUDA = 2,         /* CUDA runtime error, no device, or extension unusable */
    QMC_ERR_TIMEOUT = 3,      /* a bounded device wait gave up */
    QMC_ERR_SINGULAR = 4,     /* a Slater matrix was singular (reference: identity fallback) */
    QMC_ERR_POPULATION = 5,   /* DMC population left [N/4, 4N] */
    QMC_ERR_NONFINITE = 6,    /* NaN/Inf ratio, energy or position */
    QMC_ERR_UNSUPPORTED = 7,  /* no compiled kernel for this system shape */
    QMC_ERR_NOMEM = 8
};

/* ---- enumerations -------------------------------------------------------- */
enum { QMC_FP64 = 0, QMC_FP32_REFINE = 1 };          /* walker working precision */
enum { QMC_BASIS_GTO = 0, QMC_BASIS_STO = 1, QMC_BASIS_PW = 2 };   /* contracted Gaussians / Slater-type / plane waves */
enum { QMC_JAS_NONE = 0, QMC_JAS_PADE_F = 1, QMC_JAS_PADE_EEN = 2, QMC_JAS_HEG = 3 };
enum {
    QMC_MOVE_ALL_GAUSS = 0,   /* all-electron Gaussian, src/sampling/vmc.rs:95-119 */
    QMC_MOVE_ALL_BOX = 1,     /* all-electron uniform box of side `step` */
    QMC_MOVE_ONE_GAUSS = 2,   /* single-electron Gaussian of width `step` */
    QMC_MOVE_ONE_DRIFT = 3    /* single-electron Langevin, src/sampling/vmc.rs:339-394 */
};
enum {
    QMC_QUIRK_J2_GRAD = 1,    /* Jastrow2 gradient prefactor F/(2(1+r/F)^2 r), src/correlation/jastrow.rs:102 */
    QMC_QUIRK_J2_LAP = 2,     /* Jastrow2 per-pair Laplacian without cross terms, :110-125 */
    QMC_QUIRK_HEG_EWALD = 4,  /* electron gas: the reference's Ewald (alpha = 5/L, |n_i| <= 7, minimum
                                 image, Madelung -0.448 N / r_s), src/systems/heg.rs:526-581 */
    QMC_QUIRK_HEG_CROSS = 8   /* electron gas: cross term without the orbital factor, heg.rs:711-720 */
};

/* ---- system description (MultiWfn + EnergyCalculator data) ------------- */
/*
 * Replaces the constructors of H2MoleculeMO (src/systems/hydrogen.rs:28-35),
 * Lithium (src/systems/lithium.rs:9-19), MethaneGTO (src/systems/methane.rs:
 * 600-685) and BenzeneGTO (src/systems/benzene.rs:48-112).
 *
 * MO k = sum_a mo_coef[k*n_ao + a] * chi_a.  Electron e's Slater column is MO
 * occ[e]; a spin sector's columns follow its electrons' order (the reference's
 * STOSlaterDet uses orbital j for electron j, MethaneGTO uses MOs 0..n-1).
 * Jastrow parameters for QMC_JAS_PADE_EEN, jas[] =
 *   { b_anti, b_para, a_anti, a_para, B_0, B_1, A_0, A_1 }
 *   u = sum_{i<j} a_s r/(1+b_s r) - sum_{i,I} A_sp Z_I r/(1+B_sp r),
 *   s = spin class of the pair, sp = nuc_species[I];
 * the reference Jastrow3 is b_anti=b_para=b_ee, A=1, B_0=B_1=b_en.
 * QMC_JAS_PADE_F is u = sum_{i<j} -F/(2(1+r/F)) (Jastrow1 / Jastrow2).
 * Periodic electron gas (src/systems/heg.rs): basis_kind QMC_BASIS_PW, box_L
 * the cubic box side, n_nuc = 0, mo_coef the plane-wave vectors [n_mo][3]
 * (orbital k = e^{i k.r}), jastrow_kind QMC_JAS_HEG with jas_F = F,
 * jas[0] = form (0 Pade, 1 RPA, 2 Yukawa), jas[2]/jas[3] = antiparallel /
 * parallel amplitudes, jas[4] = Ewald alpha * L, jas[5] = reciprocal cutoff
 * |n| (one-component-plasma Ewald unless QMC_QUIRK_HEG_EWALD).  Walkers start
 * uniformly in the box; accepted moves are wrapped into it.
 * Optimisable parameters (OptimizableWfn) are jas[0..7] then rot_angle[0..n_rot-1]:
 * angle q mixes MO rot_occ[q] with MO rot_virt[q]:
 *   phi_occ <- cos(t) phi_occ + sin(t) phi_virt.
 */
typedef struct {
    int n_elec;
    const int* spins;            /* [n_elec] +1 / -1 */
    int n_nuc;
    const double* nuc_pos;       /* [n_nuc*3] */
    const double* nuc_charge;    /* [n_nuc] */
    const int* nuc_species;      /* [n_nuc] 0/1, or NULL */
    int basis_kind;
    int n_ao;
    const int* ao_nuc;           /* [n_ao] centre of each AO */
    const int* ao_l;             /* [n_ao] 0 = s, 1 = p */
    const int* ao_m;             /* [n_ao] p component 0/1/2 = x/y/z */
    const int* ao_prim_off;      /* [n_ao+1] primitive ranges */
    const double* prim_exp;
    const double* prim_coef;
    const int* prim_pow;         /* Slater-type r^n powers; NULL for Gaussians */
    int n_mo;
    const double* mo_coef;       /* [n_mo*n_ao] */
    const int* occ;              /* [n_elec] */
    int jastrow_kind;
    double jas_F;
    double jas[8];
    int n_rot;
    const int* rot_occ;
    const int* rot_virt;
    const double* rot_angle;
    int quirks;
    const int* init_nuc;         /* [n_elec] initial centre per electron, -1 = origin; NULL = all origin */
    double init_sigma;           /* width of the initial Gaussian (MultiWfn::initialize) */
    double box_L;                /* 0: open boundaries; > 0: periodic cubic box (plane-wave systems) */
    int reserved[4];
} qmc_system_desc;

/* Parameters of a sampling run (MCMCParams src/sampling/vmc.rs:13-21,
 * DDVMCParams :197-226, ISDMCParams src/sampling/is_dmc.rs:51-86). */
typedef struct {
    int n_walkers;
    int n_steps;                 /* production steps (sweeps for single-electron moves) */
    int n_burnin;
    int move_kind;               /* QMC_MOVE_* */
    double step;                 /* Gaussian width / box side */
    double tau;                  /* drift-diffusion / DMC time step */
    double max_drift;            /* |tau F| cap */
    int precision;               /* QMC_FP64 / QMC_FP32_REFINE */
    int refresh_every;           /* FP64 inverse recompute + E_L measurement period (sweeps) */
    double e_ref_damping;        /* DMC kappa */
    int fixed_node;              /* DMC: refuse sign-changing proposals (the reference accepts them) */
    int reference_diffusion;     /* DMC: move with variance 2 tau as the reference does (is_dmc.rs:218-225);
                                    0 = Hartree-unit diffusion (variance tau, drift tau grad ln psi) */
    /* VMC step adaptation (MCMCParams target_acceptance / adaptation_interval /
     * min_step_size / max_step_size, src/sampling/vmc.rs:13-21; DDVMCParams
     * :197-226).  target_acceptance > 0 turns it on: every adaptation_interval
     * steps (sweeps), through burn-in and production, the acceptance of that
     * window rescales the all-electron or Gaussian step by sqrt(rate / target)
     * (MCMCSimulation::adapt_step_size, vmc.rs:122-128) or tau by that factor
     * clamped to [0.8, 1.2] (DriftDiffusionVMC::adapt_time_step,
     * vmc.rs:397-402), then clamps it to [min_step, max_step] (0 = the
     * reference's [0.001, 0.05] for tau, no bound for the step). */
    double target_acceptance;
    int adaptation_interval;
    double min_step;
    double max_step;
    /* DMC: > 0 clamps the branching energy (E_L + E_L,old)/2 to E_ref +- branch_cut
     * (the reference branches on it unclamped, is_dmc.rs:278-302; a cut of
     * 2 / sqrt(tau) in the manner of Umrigar, Nightingale and Runge, J. Chem. Phys.
     * 99, 2865 (1993), keeps populations of trial functions with nodal E_L
     * divergences finite); 0 = the reference's branching */
    double branch_cut;
    int reserved[2];
} qmc_run_params;

typedef struct {
    double energy;
    double error;
    double autocorrelation_time;
    double acceptance_rate;
    double variance;
    int n_samples;
    int status_flags;            /* OR of: 1 singular, 2 non-finite, 4 DMC population collapse (re-initialised),
                                    8 a bounded device wait of a sweep gave up */
    double avg_population;
    double final_step;           /* VMC: the step (all-electron / Gaussian) or tau (drift) after adaptation */
    double reserved[3];
} qmc_run_result;

typedef struct qmc_ctx_s* qmc_ctx_t;
typedef struct qmc_sys_s* qmc_sys_t;
typedef struct qmc_walkers_s* qmc_walkers_t;
typedef struct qmc_batch_s* qmc_batch_t;

/* ---- context --------------------------------------------------------------- */
int qmc_init(int device, qmc_ctx_t* out);
int qmc_destroy(qmc_ctx_t ctx);
const char* qmc_status_string(int status);
int qmc_version(void);

/* ---- systems ------------------------------------------------------------- */
/* Builds device-ready tables from the description (replaces the reference
 * constructors listed above).  QMC_ERR_UNSUPPORTED if no kernel is compiled
 * for the (n_elec, n_up, n_nuc, basis, Jastrow) shape. */
int qmc_system_create(qmc_ctx_t ctx, const qmc_system_desc* desc, qmc_sys_t* out);
/* Validates a description without touching a device; *shape (may be NULL)
 * receives the compiled kernel shape it maps to. */
int qmc_system_check(const qmc_system_desc* desc, int* shape);
int qmc_system_destroy(qmc_sys_t sys);
/* OptimizableWfn::num_params/get_params/set_params, src/wavefunction/traits.rs:98-106 */
int qmc_system_num_params(qmc_sys_t sys, int* P);
int qmc_system_get_params(qmc_sys_t sys, double* p, int P);
int qmc_system_set_params(qmc_sys_t sys, const double* p, int P);
/* ForceCalculator::num_nuclei/set_nuclei, src/sampling/traits.rs:22-31 */
int qmc_system_set_nuclei(qmc_sys_t sys, const double* R, int n_nuc);

/* ---- batched evaluation (MultiWfn / EnergyCalculator / OptimizableWfn /
 *      ForceCalculator methods for W configurations at once) ---------------- */
/* MultiWfn::evaluate/derivative/laplacian (src/wavefunction/traits.rs:53-59)
 * and EnergyCalculator::local_energy (src/sampling/traits.rs:6-8).
 * precision QMC_FP64 evaluates in double; QMC_FP32_REFINE evaluates orbitals,
 * determinants and E_L in single precision (the moving-walker form).
 * Any output pointer may be NULL. */
int qmc_eval_batch(qmc_sys_t sys, int W, const double* pos, int precision,
                   double* logabs, int* sign, double* grad_ln, double* lap_over_psi,
                   double* e_local);

/* OptimizableWfn::log_derivatives (src/wavefunction/traits.rs:114;
 * src/systems/methane.rs:1212-1219, benzene.rs:748-755): O [W x P] plus
 * E_L [W]; dEL [W x P] = d E_L / d p (the derivative of
 * EnergyCalculator::local_energy, src/systems/methane.rs:1154-1182, in each
 * optimisable parameter; analytic: through the Jastrow's gradient and
 * Laplacian and, for MO-rotation angles, through the Slater inverse);
 * optionally the FP64 compensated SR sums over the batch
 * (src/sampling/sr_optimize.rs:176-246): S [P x P] = <O O^T> - <O><O>^T,
 * f [P] = <E O> - <E><O>, e_mean (any output may be NULL).  Systems with the
 * Jastrow3 factor; benzene without MO-rotation angles (P = 8). */
int qmc_logderiv_batch(qmc_sys_t sys, int W, const double* pos, double* O, double* e_local,
                       double* dEL, double* S, double* f, double* e_mean);

/* ForceCalculator::hellmann_feynman_force and wfn_nuclear_gradient
 * (src/sampling/traits.rs:38,50; src/systems/methane.rs:1007-1101,1241-1272):
 * F_hf [W x n_nuc x 3], omega = d ln|psi| / dR_I [W x n_nuc x 3].
 * Benzene has the Hellmann-Feynman force only (src/systems/benzene.rs:828-858;
 * its wfn_nuclear_gradient is the trait's unimplemented default): omega must
 * be NULL for it (QMC_ERR_UNSUPPORTED otherwise). */
int qmc_forces_batch(qmc_sys_t sys, int W, const double* pos, double* F_hf, double* omega);

/* ---- resident walker ensembles (the sampler state: Vec<MCMCState>,
 *      DDWalkerState, ISDMCWalker in the reference) ------------------------- */
int qmc_walkers_create(qmc_sys_t sys, int W, int precision, qmc_walkers_t* out);
int qmc_walkers_destroy(qmc_walkers_t wk);
/* MultiWfn::initialize for every walker, seeded (tag 3 draws). */
int qmc_walkers_init(qmc_walkers_t wk, uint64_t seed);
/* Host <-> device positions (W x n_elec x 3, caller order). */
int qmc_walkers_set_positions(qmc_walkers_t wk, const double* pos);
int qmc_walkers_get_positions(qmc_walkers_t wk, double* pos);
/* FP64 rebuild of every walker's inverse Slater matrices and log|psi| from its
 * positions, plus the FP64 local energy.  e_local [W] may be NULL (kept on
 * the device); e_sum receives the FP64 compensated sum (may be NULL). */
int qmc_walkers_refresh(qmc_walkers_t wk, double* e_local, double* e_sum);
/* FP64 rebuild of the inverse Slater matrices, sign and log|psi| only: the
 * state a sweep needs after qmc_walkers_set_positions (the reference's
 * DDWalkerState::refresh, src/sampling/vmc.rs:243-276, without the drift).  The
 * stored E_L values are unspecified until the next qmc_walkers_refresh. */
int qmc_walkers_rebuild_inverse(qmc_walkers_t wk);
/* n_sweeps Monte Carlo steps for all walkers (one launch):
 * src/sampling/vmc.rs:95-119 (all-electron), :339-394 (single-electron).
 * Sweep indices step0 .. step0+n_sweeps-1 key the random stream.
 * accepted (may be NULL) receives the number of accepted proposals. */
int qmc_walkers_sweep(qmc_walkers_t wk, int move_kind, int n_sweeps, uint64_t step0,
                      double step, double tau, double max_drift, uint64_t seed,
                      long long* accepted);
/* Per-walker E_L [W] (device values from the last refresh) and logabs/sign. */
int qmc_walkers_get_state(qmc_walkers_t wk, double* logabs, int* sign, double* e_local);
/* Bitwise OR of the per-walker status flags raised since the last call
 * (1 singular, 2 non-finite, 8 a bounded device wait of a sweep gave up);
 * cleared on read. */
int qmc_walkers_status(qmc_walkers_t wk, int* flags);

/* Walker set with room for `capacity` walkers (DMC populations grow and
 * shrink); W is the initial population. */
int qmc_walkers_create_dmc(qmc_sys_t sys, int W, int capacity, int precision, qmc_walkers_t* out);
/* Current population size. */
int qmc_walkers_count(qmc_walkers_t wk, int* W);
/* One IS-DMC step (src/sampling/is_dmc.rs:208-302; branch_cut as in
 * qmc_run_params, 0 = the reference's branching): one drift-diffusion sweep
 * per walker made with the reference-convention move at tau_move (variance
 * 2 tau_move, drift 2 tau_move grad ln psi; tau_move = tau / 2 is the
 * Hartree-unit projector, tau_move = tau the reference's), fixed-node
 * rejection when fixed_node, E_L after the sweep (in
 * the walkers' precision, FP64 when fp64_measure), copies
 * m = min(floor(exp(tau (e_ref - (E_L + E_old)/2)) + xi), 3) with an FP64
 * log-weight and a tag-4 Philox xi per (walker slot, step), and an
 * order-stable on-device compaction.  *n_new receives the new population
 * (0 = collapse), *e_mean its mean E_L.  QMC_ERR_POPULATION if the new
 * population exceeds the capacity (the population is then left unchanged). */
int qmc_walkers_dmc_step(qmc_walkers_t wk, double tau, double tau_move, double max_drift, int fixed_node,
                         double e_ref, uint64_t seed, uint64_t step, int fp64_measure, double branch_cut, int* n_new,
                         double* e_mean);

/* ---- drivers --------------------------------------------------------------- */
/* VMC run: MCMCSimulation::run (src/sampling/vmc.rs:69-92) for all-electron
 * moves, DriftDiffusionVMC::run (:405-484) for single-electron moves.  With
 * single-electron moves E_L is measured (FP64) every refresh_every sweeps.
 * energies (may be NULL) receives the per-measurement mean energies
 * (capacity n_steps). */
int qmc_vmc_run(qmc_sys_t sys, const qmc_run_params* params, uint64_t seed,
                qmc_run_result* result, double* energies);

/* ImportanceSampledDMC::run (src/sampling/is_dmc.rs:385-553) energy part:
 * target population n_walkers (capacity 4x), n_burnin + n_steps steps of
 * qmc_walkers_dmc_step, E_ref = <E_L> - kappa ln(N / N_target) / tau,
 * collapse -> re-initialisation; energy = mean of the per-step mixed
 * estimates, error by blocking (is_dmc.rs:556-607).  FP32 walkers measure
 * E_L in FP64 every refresh_every steps. */
int qmc_dmc_run(qmc_sys_t sys, const qmc_run_params* params, uint64_t seed, qmc_run_result* result,
                double* energies);
/* ImportanceSampledDMC::run with its force estimators (src/sampling/is_dmc.rs:
 * 303-380, 479-485, 520-534), [n_nuc x 3] each, in the reference's
 * hellmann_feynman_force convention (src/systems/methane.rs:1241-1272):
 * forces_vmc   = <F_HF> of a separate VMC run: min(n_walkers, 50) walkers,
 *                all-electron Gaussian moves of width 0.5 (single-electron
 *                sweeps of that width for benzene), n_vmc_equilibrate steps,
 *                then max(1, n_vmc_force_samples / walkers) rounds of five
 *                steps, each recording every walker;
 * forces_mixed = <F_HF> over every walker of every production step of the
 *                DMC run (the run of qmc_dmc_run with the same seed);
 * forces_extrapolated = 2 forces_mixed - forces_vmc.
 * The electron sums run on the device (FP64, compensated, per step). */
int qmc_dmc_run_forces(qmc_sys_t sys, const qmc_run_params* params, int n_vmc_equilibrate,
                       int n_vmc_force_samples, uint64_t seed, qmc_run_result* result, double* energies,
                       double* forces_mixed, double* forces_vmc, double* forces_extrapolated);

/* ---- single-electron ratio (MultiWfn evaluate twice, src/sampling/vmc.rs:356-370) ---- */
/* ratio[w] = psi(R_w with electron e at r_new[w]) / psi(R_w) for W
 * configurations pos (W x n_elec x 3, caller order; e in caller order), and
 * grad_ln_new[w] (may be NULL) = grad_e ln psi at the moved configuration,
 * the drift of the reference's Langevin proposal.  FP64 evaluation. */
int qmc_ratio_batch(qmc_sys_t sys, int W, const double* pos, int e, const double* r_new, double* ratio,
                    double* grad_ln_new);

/* ---- algorithmic counts (no reference counterpart; the benchmark's roofline) ---- */
typedef struct {
    double sweep_flops_per_move;  /* FP32 operations of one single-electron Gaussian proposal
                                     (transcendentals count one) at the given acceptance */
    double sweep_state_bytes;     /* walker state read + written by one sweep launch, per walker */
    double refresh_flops;         /* FP64-class operations of one refresh, per walker */
    double refresh_bytes;         /* HBM bytes of one refresh, per walker (state + two-pass scratch) */
    double reserved[4];
} qmc_roofline_counts;
/* Host-only (no device needed): the counts for a system description and a
 * walker precision. */
int qmc_roofline_model(const qmc_system_desc* desc, int precision, double acceptance, qmc_roofline_counts* out);

/* ---- uneven batches (no reference counterpart: rust_qmc runs one system
 * per process, src/main.rs) ---------------------------------------------------
 * A batch binds walker sets of one context -- any mix of systems, shapes,
 * precisions and sizes -- and advances them together: one sweep launch and
 * one refresh (one or two launches) per (shape, precision) class over
 * (system, walker tile) pairs, the class launches running concurrently inside
 * one CUDA graph per step.
 * Walker set i of a batch driven with `seed` draws from the Philox key
 * qmc_batch_system_seed(seed, i) (SplitMix64 of seed + (i+1) * 0x9E3779B97F4A7C15),
 * so a batched sweep of set i equals qmc_walkers_sweep of that set with that
 * key.  A walker set may belong to several batches (not at the same time on
 * different streams); destroying it while bound defers its release until the
 * last batch binding it is destroyed. */
uint64_t qmc_batch_system_seed(uint64_t seed, int i);
/* Binds n distinct walker sets of ctx (n >= 1). */
int qmc_batch_create(qmc_ctx_t ctx, int n, const qmc_walkers_t* walkers, qmc_batch_t* out);
int qmc_batch_destroy(qmc_batch_t batch);
/* n_sweeps single-electron sweeps (QMC_MOVE_ONE_GAUSS / QMC_MOVE_ONE_DRIFT) of
 * every walker set, sweep counters step0 .. step0 + n_sweeps - 1. */
int qmc_batch_sweep(qmc_batch_t batch, int move_kind, int n_sweeps, uint64_t step0, double step, double tau,
                    double max_drift, uint64_t seed);
/* FP64 refresh of every walker set (inverse, log|psi|, E_L) and the mean E_L
 * of each set, e_mean[n] (may be NULL). */
int qmc_batch_refresh(qmc_batch_t batch, double* e_mean);
/* n_steps graph-captured steps: sweeps_per_step sweeps, then the FP64
 * refresh; e_series[n_steps][n] (may be NULL) receives the per-step mean E_L
 * of every set.  Step k sweeps with counters step0 + k * sweeps_per_step + j. */
int qmc_batch_run_steps(qmc_batch_t batch, int move_kind, int n_steps, int sweeps_per_step, uint64_t step0,
                        double step, double tau, double max_drift, uint64_t seed, double* e_series);
/* VMC of n_sys systems in one batch (W[i] walkers each, params->n_walkers
 * ignored; single-electron moves; fixed step: QMC_ERR_UNSUPPORTED with
 * target_acceptance > 0): system i follows exactly the schedule of
 * qmc_vmc_run(systems[i], params, qmc_batch_system_seed(seed, i)) and
 * per_sys[i] holds its result.  energies (may be NULL) receives
 * [ceil(n_steps / refresh_every)][n_sys] per-measurement means. */
int qmc_batch_run(qmc_ctx_t ctx, int n_sys, const qmc_sys_t* systems, const int* W, const qmc_run_params* params,
                  uint64_t seed, qmc_run_result* per_sys, double* energies);

/* ---- timing helpers (no reference counterpart; used by the benchmark) ---- */
/* Records CUDA event `slot` (0..15) on the context's stream. */
int qmc_ctx_event_record(qmc_ctx_t ctx, int slot);
/* Milliseconds between two recorded events (synchronises on `b`). */
int qmc_ctx_event_elapsed(qmc_ctx_t ctx, int a, int b, float* ms);
int qmc_ctx_synchronize(qmc_ctx_t ctx);
/* Writes a device buffer larger than L2 to evict cached walker state. */
int qmc_ctx_flush_l2(qmc_ctx_t ctx);
/* Counts of kernel launches issued by this context since creation. */
int qmc_ctx_launch_count(qmc_ctx_t ctx, long long* n);
/* Measured FMA throughput of this GPU's CUDA cores (FP32 and FP64), the
 * compute roofline of the walker kernels. */
int qmc_ctx_measure_peaks(qmc_ctx_t ctx, double* fp32_tflops, double* fp64_tflops);
/* Page-locked host buffers for asynchronous host<->device copies. */
int qmc_host_alloc(size_t bytes, void** out);
int qmc_host_free(void* p);

/* ---- allocation-free reduction (no counterpart in the reference) -------- */
/* The FP64 compensated SR walker sums of qmc_logderiv_batch (sum E, sum E^2,
 * sum O_p, sum E O_p, sum O_p O_q for p <= q, in that order; deterministic)
 * over inputs that are already on the device, for callers that cannot
 * allocate device memory: code between cudaStreamBeginCapture and
 * cudaStreamEndCapture, hosts whose device memory belongs to another
 * framework's allocator, latency-critical loops that cannot absorb
 * cudaFree's implicit synchronisation.  It calls no allocator: its scratch
 * is a static 512 KiB device array that every GPU loading the library holds
 * until the process exits.
 *   d_E [W], d_O [W x P] row-major, d_sums [2 + 2P + P(P+1)/2]: device pointers.
 *   stream: a cudaStream_t, or NULL for the legacy default stream.
 * Limits: P <= QMC_NOALLOC_MAX_PARAMS and 2 (2 + 2P + P(P+1)/2) ceil(W/256)
 * <= 65536 (for P = 12, W <= 80640); larger sizes return QMC_ERR_ARG and a
 * message on stderr.  The first call on each device looks up the scratch's
 * device address (set-up); make that first call before any stream capture.
 * All calls share the scratch: calls that overlap on the GPU (other streams,
 * other host threads on the same device) race and must be serialised. */
#define QMC_NOALLOC_MAX_PARAMS 16
int qmc_sr_sums_noalloc(const double* d_E, const double* d_O, int W, int P, double* d_sums, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* QMC_GB300_H */

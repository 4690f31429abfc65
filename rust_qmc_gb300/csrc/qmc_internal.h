// qmc_internal.h -- host-side representation of a system and the launch
// interface between the C ABI (qmc_api.cpp) and the CUDA kernels
// (qmc_kernels.cu).  Not part of the public ABI.
#pragma once
#include <cstdint>
#include <vector>
#include <cuda_runtime.h>

namespace qmc {

// Kernel shapes compiled into the library.  A shape fixes the electron
// counts and nucleus count at compile time so per-walker arrays live in
// registers / shared memory with static indices.
enum Shape { SHAPE_H2 = 0, SHAPE_LI = 1, SHAPE_CH4 = 2, SHAPE_CH4MIN = 3, SHAPE_C6H6 = 4, SHAPE_HEG54 = 5, SHAPE_COUNT = 6 };

// A basis shell: primitives shared by up to two s-type AOs and one p triplet
// (the SP shells of 6-31G share exponents between 2s and 2p; Li's STO-7G 1s
// and 2s share exponents and powers).
struct HostShell {
    int nuc;
    std::vector<double> exps;
    std::vector<int> pows;
    int s_ao[2] = {-1, -1};              // caller AO index of the s-type AOs
    std::vector<double> s_coef[2];
    int p_ao[3] = {-1, -1, -1};          // caller AO index of px, py, pz
    std::vector<double> p_coef;
};

struct HostSys {
    int shape = -1;
    int N = 0, n_up = 0, n_dn = 0, n_nuc = 0, n_ao = 0, n_mo = 0;
    std::vector<int> perm;               // internal electron index -> caller index
    std::vector<int> spins;              // caller order
    std::vector<double> R;               // [n_nuc*3]
    std::vector<double> Z;
    std::vector<int> species;
    int basis = 0;
    std::vector<HostShell> shells;       // sorted by nucleus
    std::vector<int> ao_int;             // caller AO -> internal AO index (shell order)
    std::vector<double> C0;              // caller MO coefficients [n_mo*n_ao] (caller AO order)
    std::vector<int> occ;                // caller order
    int jk = 0;
    double F = 1.0;
    double jas[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    std::vector<int> rot_occ, rot_virt;
    std::vector<double> rot_angle;
    int quirks = 0;
    std::vector<int> init_nuc;           // caller order
    double init_sigma = 0.5;
    double v_nn = 0.0;
    double box_L = 0.0;                  // periodic electron gas: box side
    std::vector<double> kvec;            // periodic electron gas: [n_mo*3] orbital wave vectors
    int version = 0;                     // bumped when parameters or nuclei change
    // cached device copies of the system table per arithmetic type:
    // [0] FP64, [1] FP32, [2] float-float
    mutable void* dev_table[3] = {nullptr, nullptr, nullptr};
    mutable int dev_table_version[3] = {-1, -1, -1};

    int n_params() const { return 8 + (int)rot_occ.size(); }
    // Effective (rotated) MO coefficients in caller AO order.
    std::vector<double> effective_mo() const;
    // d phi_k / d theta_q coefficient rows, one per rotation.
    std::vector<double> rotation_derivative_rows() const;
};

// Device-resident walker arrays, structure-of-arrays with stride Wcap.
struct DevWalkers {
    int W = 0, Wcap = 0;
    int prec = 0;                        // 0 FP64, 1 FP32 storage
    void* pos = nullptr;                 // [N*3][Wcap]
    void* dinv = nullptr;                // [2][nmax*nmax][Wcap]
    double* logabs = nullptr;            // [Wcap]
    int* sign = nullptr;                 // [Wcap]
    double* el = nullptr;                // [Wcap]
    int* flags = nullptr;                // [1] status bits (OR)
    unsigned long long* acc = nullptr;   // [1] accepted-move counter
    double* partial = nullptr;           // reduction scratch
    int partial_cap = 0;
    int fixed_node = 0;                  // sweeps refuse sign-changing proposals (DMC)
    float2* rows = nullptr;              // two-pass refresh scratch [N][row quantities][Wcap] (FP32 walkers)
    unsigned* chunk_done = nullptr;      // [Wcap / 32] chunked sweeps: chunks published per 32-walker group (FP32 walkers)
    float* chunk_jc = nullptr;           // chunked Gaussian sweeps: pair cache + one-body terms between chunks (allocated on first use)
};

// Device buffers of the DMC branching step (population control).
struct DevBranch {
    int cap = 0;
    int* counts = nullptr;               // [cap] copies per walker
    int* offsets = nullptr;              // [cap] exclusive scan
    double* el_old = nullptr;            // [cap] E_L before the sweep
    double* stats = nullptr;             // [4] total copies, sum m E (compensated), flags
};

struct MeasureOut {
    double* grad = nullptr;              // [W][N][3] internal order
    double* lap = nullptr;               // [W][N]
    double* O = nullptr;                 // [W][P]
    double* fhf = nullptr;               // [W][n_nuc][3]
    double* omega = nullptr;             // [W][n_nuc][3]
    double* dEL = nullptr;               // [W][P] d E_L / dp: rotation columns 8.. (with O)
    // only the inverse, sign and log|psi| are wanted (E_L may be skipped)
    bool inverse_only = false;
};

int nmax_of_shape(int shape);
// Bytes per walker of the two-pass refresh scratch (0: the shape has none).
size_t refresh_rows_bytes(int shape);
// Scalars per walker in the inverse-matrix block (2 x nmax^2, doubled for
// complex determinants).
int dinv_elems_of_shape(int shape);
// True when the system's shells match the compile-time 9-function CH4 layout.
bool layout_matches_ch4min(const HostSys& hs);

// Launchers (return a qmc status).  compute_prec: 0 double, 1 float.
int launch_init(const HostSys& hs, DevWalkers& dw, uint64_t seed, cudaStream_t st);
int launch_measure(const HostSys& hs, DevWalkers& dw, int compute_prec, bool write_state,
                   const MeasureOut& out, cudaStream_t st);
int launch_sweep(const HostSys& hs, DevWalkers& dw, int move_kind, int n_sweeps, uint64_t step0,
                 double step, double tau, double max_drift, uint64_t seed, cudaStream_t st);
// FP64 compensated sums.  Sums column c of X (row-major [W][ncol]) into
// out[c]; when `products` is set also out[ncol + ...] = sum of the pairwise
// products used by the SR matrices (see qmc_kernels.cu).
int launch_walker_sum(const double* X, int W, int ncol, double* d_out, double* d_scratch,
                      int scratch_cap, cudaStream_t st);
int launch_sr_sums(const double* E, const double* O, int W, int P, double* d_out,
                   double* d_scratch, int scratch_cap, cudaStream_t st);
int launch_flush(void* buf, size_t bytes, cudaStream_t st);
// Sum over the W walkers of the Hellmann-Feynman electron-nucleus forces into
// d_out[3 n_nuc] (FP64, compensated); d_nuc = [n_nuc][4] (x, y, z, Z); the
// scratch holds hf_force_scratch_doubles(W, n_nuc) doubles.
size_t hf_force_scratch_doubles(int W, int n_nuc);
int launch_sum_partials(const double* partial, int nblk, int nrows, double* out, cudaStream_t st);
// Jastrow3 parameter log-derivatives d_O [W][P] (columns 0..7; skipped when
// null) from the walkers' positions; d_par = jas[8], d_nuc = [n_nuc][5]
// (x, y, z, Z, species 0 or 1 -- two species only, as build_hostsys
// enforces).  With d_grad ([W][N][3] grad ln|psi|, internal order) also the
// Jastrow-parameter derivatives of E_L into d_dEL [W][P] (columns 0..7).
int launch_jastrow3_logderiv(const DevWalkers& dw, int N, int n_up, int n_nuc, const double* d_nuc,
                             const double* d_par, int P, double* d_O, cudaStream_t st,
                             const double* d_grad = nullptr, double* d_dEL = nullptr);
// Per-walker Hellmann-Feynman forces d_out [W][n_nuc][3] (electron order is
// irrelevant: the force sums over all electrons).
int launch_hf_force_walkers(const DevWalkers& dw, int N, int n_nuc, const double* d_nuc, double* d_out,
                            cudaStream_t st);
int launch_hf_force_sum(const DevWalkers& dw, int N, int n_nuc, const double* d_nuc, double* d_partial,
                        size_t partial_cap, double* d_out, cudaStream_t st);
// DMC branching (src/sampling/is_dmc.rs:278-302): copies per walker from the
// FP64 log-weight, exclusive scan, order-stable gather into `dst`.  e_cut > 0
// clamps the branching energy (E_L + E_old)/2 to e_ref +- e_cut.
// stats[0] = new population, stats[1] = sum of copies x E_L, stats[2] = flags.
int launch_branch(DevWalkers& src, DevWalkers& dst, DevBranch& br, int n_elec, int nmax, double e_ref,
                  double tau, double e_cut, uint64_t seed, uint64_t step, cudaStream_t st);

// ---------------------------------------------------------------------------
// Uneven batches: many systems, each with its own walker set, advanced by a
// few launches per shape class over a list of (system, walker tile).
// ---------------------------------------------------------------------------
#if defined(__CUDACC__)
#define QMC_HD __host__ __device__
#else
#define QMC_HD
#endif

// Philox key of system s in a batch driven with `seed` (SplitMix64 of the
// seed offset by the golden-ratio increment per system): a batched sweep of
// system s is the standalone sweep of its walker set with this seed.
QMC_HD inline uint64_t batch_system_seed(uint64_t seed, int s) {
    uint64_t z = seed + 0x9E3779B97F4A7C15ull * (uint64_t)(s + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// One system of a batch (device-resident).
struct BatchRec {
    const void* tab_d = nullptr;         // system table, FP64 form (shape-specific type)
    const void* tab_s = nullptr;         // system table in the walkers' precision
    const void* ktab = nullptr;          // reciprocal-space table (electron gas), else null
    void* pos = nullptr;
    void* dinv = nullptr;
    int* sign = nullptr;
    double* logabs = nullptr;
    double* el = nullptr;
    unsigned long long* acc = nullptr;
    int* flags = nullptr;
    int W = 0, Wcap = 0;
    int index = 0;                       // position in the batch (selects the Philox key)
    int fixed_node = 0;
    float2* rows = nullptr;              // two-pass refresh scratch of FP32 walkers
};

// A tile: walkers [w0, w0 + tile width) of record `rec`; tiles of one record
// are contiguous in the list.
struct BatchTile {
    int rec;
    int w0;
};

// Per-call scalars, read by the kernels from device memory so that a
// captured graph replays with new values and advances its own step counter.
struct BatchCtl {
    unsigned long long step = 0;         // sweep counter of the next sweep
    unsigned long long seed = 0;
    double step_size = 0, tau = 0, max_drift = 0;
    int n_sweeps = 0;
    int row = 0;                         // energy-series row of the next measurement
};

// One shape class of a batch.
struct BatchClass {
    int shape = -1;
    int prec = 0;
    const BatchTile* tiles = nullptr;    // device
    int ntiles = 0;
    const BatchRec* recs = nullptr;      // device, indexed by BatchTile::rec
    int nrec = 0;
    const int* tile_begin = nullptr;     // device [nrec + 1]
    double* tile_partial = nullptr;      // device [ntiles][2]
    int grid_measure = 0;                // persistent refresh grid of the thread-per-walker shapes
                                         // (0: one block per tile); other launches: one block per tile
};

// Walkers per tile for a shape: threads per block for the thread-per-walker
// shapes, a multiple of the warps per sweep block for the warp-per-walker ones.
int batch_tile_width(int shape);
// The launches of one class; `ctl` is device-resident.
int launch_batch_sweep(const BatchClass& bc, int move_kind, const BatchCtl* ctl, cudaStream_t st);
int launch_batch_measure(const BatchClass& bc, cudaStream_t st);
// Resident blocks per SM of the class's batch kernels (occupancy query).
int batch_occupancy(int shape, int prec, int move_kind, bool measure);
// Device tables of a system for batched launches (cached in the HostSys).
int batch_tables(const HostSys& hs, int prec, BatchRec& rec);
// Per-system mean E_L of the class: sum of its tiles' partials / W, written to
// series[ctl->row * n_total + rec.index].
int launch_batch_energy(const BatchClass& bc, const BatchCtl* ctl, double* series, int n_total, cudaStream_t st);
// ctl->step += n_sweeps, ctl->row += 1 (one thread; ends a captured step).
int launch_batch_advance(BatchCtl* ctl, cudaStream_t st);

// Algorithmic counts of the walker kernels (qmc_roofline.cpp): [0] sweep
// operations per proposal, [1] sweep state bytes per walker and launch,
// [2] refresh operations per walker, [3] refresh HBM bytes per walker.
void roofline_counts(const HostSys& hs, int prec, double acceptance, double out[4]);

extern long long g_launch_count;

}  // namespace qmc

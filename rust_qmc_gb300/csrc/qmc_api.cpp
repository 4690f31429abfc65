// qmc_api.cpp -- C ABI of libqmc_gb300 (declared in include/qmc.h): context,
// system tables, resident walker ensembles, batched evaluation and the VMC
// driver.  All numerical work runs in the CUDA kernels of qmc_kernels.cu;
// this file only validates arguments, lays data out for the device and
// orchestrates launches.  There is no CPU fallback: without a usable CUDA
// device every entry point that needs one returns QMC_ERR_CUDA.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <map>
#include <new>
#include <vector>
#include <cuda_runtime.h>
#include "../../include/qmc.h"
#include "qmc_internal.h"

using namespace qmc;

namespace qmc {
int launch_step_all_recorded(const HostSys& hs, DevWalkers& dw, int move_kind, int n, uint64_t s0, double step,
                             uint64_t seed, double* partial, cudaStream_t st);
int launch_sum_partials(const double* partial, int nblk, int nrows, double* out, cudaStream_t st);
int launch_scatter_positions(const double* src, DevWalkers& dw, const int* d_perm, int N, cudaStream_t st);
int launch_gather_positions(const DevWalkers& dw, double* dst, const int* d_perm, int N, cudaStream_t st);
int measure_fma_peak(int fp64, double* tflops, cudaStream_t st);
}

struct qmc_ctx_s {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[16] = {};
    void* flush_buf = nullptr;
    size_t flush_bytes = 0;
    long long launches0 = 0;
    int n_children = 0;                    // live systems
    bool released = false;                 // qmc_destroy called while systems were alive
};

struct qmc_walkers_s;

struct qmc_sys_s {
    qmc_ctx_s* ctx = nullptr;
    HostSys hs;
    int* d_perm = nullptr;                 // internal -> caller electron index (device)
    qmc_walkers_s* scratch[2] = {nullptr, nullptr};   // batch-evaluation walker sets per precision
    int n_children = 0;                    // live caller-owned walker sets
    bool released = false;                 // qmc_system_destroy called while walker sets were alive
};

struct qmc_walkers_s {
    qmc_sys_s* sys = nullptr;
    DevWalkers dw;
    DevWalkers alt;                        // DMC ping-pong population buffer
    DevBranch br;
    double* d_stage = nullptr;             // caller-order positions [W][N][3]
    double* d_out = nullptr;               // generic device output scratch
    size_t d_out_cap = 0;
    unsigned long long acc_host = 0;
    int n_batches = 0;                     // live batches that bind this walker set
    bool released = false;                 // qmc_walkers_destroy called while bound
};

namespace {

int cuda_rc(cudaError_t e) {
    if (e == cudaSuccess) return QMC_OK;
    std::fprintf(stderr, "qmc_gb300: %s\n", cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? QMC_ERR_NOMEM : QMC_ERR_CUDA;
}

#define CK(x) do { int _rc = (x); if (_rc) return _rc; } while (0)
#define CU(x) do { cudaError_t _e = (x); if (_e != cudaSuccess) return cuda_rc(_e); } while (0)

// Build the device-ready host description; validates every field.
// Periodic electron gas: plane-wave orbitals e^{i k.r}; mo_coef holds the
// wave vectors [n_mo][3] (src/systems/heg.rs:119-170).
int build_hostsys_pw(const qmc_system_desc* d, HostSys& hs) {
    if (!(d->box_L > 0) || d->n_mo <= 0 || !d->mo_coef || !d->occ || d->jastrow_kind != QMC_JAS_HEG) return QMC_ERR_ARG;
    if (d->jas_F <= 0 || d->jas[0] < 0 || d->jas[0] > 2) return QMC_ERR_ARG;
    if (!(d->quirks & 4) && !(d->jas[4] > 0 && d->jas[5] >= 1 && d->jas[5] <= 13)) return QMC_ERR_ARG;
    hs.basis = QMC_BASIS_PW;
    hs.box_L = d->box_L;
    hs.n_mo = d->n_mo;
    hs.kvec.assign(d->mo_coef, d->mo_coef + 3 * (size_t)d->n_mo);
    hs.occ.assign(d->occ, d->occ + hs.N);
    for (int e = 0; e < hs.N; ++e) if (hs.occ[e] < 0 || hs.occ[e] >= hs.n_mo) return QMC_ERR_ARG;
    hs.jk = d->jastrow_kind;
    hs.F = d->jas_F;
    for (int i = 0; i < 8; ++i) hs.jas[i] = d->jas[i];
    hs.quirks = d->quirks;
    hs.init_nuc.assign(hs.N, -1);
    hs.init_sigma = d->init_sigma;
    hs.shape = -1;
    if (hs.N == 54 && hs.n_up == 27) hs.shape = SHAPE_HEG54;
    return hs.shape < 0 ? QMC_ERR_UNSUPPORTED : QMC_OK;
}

int build_hostsys(const qmc_system_desc* d, HostSys& hs) {
    if (!d || d->n_elec <= 0 || d->n_elec > 64 || !d->spins) return QMC_ERR_ARG;
    if (d->basis_kind == QMC_BASIS_PW) {
        hs = HostSys();
        hs.N = d->n_elec;
        hs.spins.assign(d->spins, d->spins + hs.N);
        for (int e = 0; e < hs.N; ++e) {
            if (hs.spins[e] != 1 && hs.spins[e] != -1) return QMC_ERR_ARG;
            if (hs.spins[e] > 0) hs.n_up++; else hs.n_dn++;
        }
        for (int sig = 0; sig < 2; ++sig)
            for (int e = 0; e < hs.N; ++e)
                if ((hs.spins[e] > 0) == (sig == 0)) hs.perm.push_back(e);
        return build_hostsys_pw(d, hs);
    }
    if (d->n_nuc <= 0 || d->n_nuc > 32) return QMC_ERR_ARG;
    if (!d->nuc_pos || !d->nuc_charge || d->n_ao <= 0 || !d->ao_nuc || !d->ao_l || !d->ao_m || !d->ao_prim_off) return QMC_ERR_ARG;
    if (!d->prim_exp || !d->prim_coef || d->n_mo <= 0 || !d->mo_coef || !d->occ) return QMC_ERR_ARG;
    if (d->box_L != 0.0) return QMC_ERR_UNSUPPORTED;
    if (d->basis_kind != QMC_BASIS_GTO && d->basis_kind != QMC_BASIS_STO) return QMC_ERR_ARG;
    if (d->jastrow_kind < 0 || d->jastrow_kind > 2) return QMC_ERR_ARG;   // QMC_JAS_HEG needs plane waves
    if (d->n_rot < 0 || d->n_rot > 16 || (d->n_rot && (!d->rot_occ || !d->rot_virt || !d->rot_angle))) return QMC_ERR_ARG;
    hs = HostSys();
    hs.N = d->n_elec;
    hs.spins.assign(d->spins, d->spins + hs.N);
    for (int e = 0; e < hs.N; ++e) {
        if (hs.spins[e] != 1 && hs.spins[e] != -1) return QMC_ERR_ARG;
        if (hs.spins[e] > 0) hs.n_up++; else hs.n_dn++;
    }
    for (int sig = 0; sig < 2; ++sig)
        for (int e = 0; e < hs.N; ++e)
            if ((hs.spins[e] > 0) == (sig == 0)) hs.perm.push_back(e);
    hs.n_nuc = d->n_nuc;
    hs.R.assign(d->nuc_pos, d->nuc_pos + 3 * hs.n_nuc);
    hs.Z.assign(d->nuc_charge, d->nuc_charge + hs.n_nuc);
    for (int I = 0; I < hs.n_nuc; ++I) {
        int sp = d->nuc_species ? d->nuc_species[I] : 0;
        if (sp < 0 || sp > 1) return QMC_ERR_ARG;
        hs.species.push_back(sp);
    }
    hs.basis = d->basis_kind;
    hs.n_ao = d->n_ao;
    hs.n_mo = d->n_mo;
    int np = d->ao_prim_off[hs.n_ao];
    if (d->ao_prim_off[0] != 0 || np <= 0) return QMC_ERR_ARG;
    for (int a = 0; a < hs.n_ao; ++a) {
        if (d->ao_prim_off[a + 1] <= d->ao_prim_off[a]) return QMC_ERR_ARG;
        if (d->ao_nuc[a] < 0 || d->ao_nuc[a] >= hs.n_nuc) return QMC_ERR_ARG;
        if (d->ao_l[a] < 0 || d->ao_l[a] > 1 || d->ao_m[a] < 0 || d->ao_m[a] > 2) return QMC_ERR_ARG;
        if (d->basis_kind == QMC_BASIS_STO && d->ao_l[a] != 0) return QMC_ERR_ARG;
    }
    // group AOs into shells (same centre, exponents and powers)
    std::vector<int> used(hs.n_ao, 0);
    auto prim_exps = [&](int a) { return std::vector<double>(d->prim_exp + d->ao_prim_off[a], d->prim_exp + d->ao_prim_off[a + 1]); };
    auto prim_pows = [&](int a) {
        if (!d->prim_pow) return std::vector<int>(d->ao_prim_off[a + 1] - d->ao_prim_off[a], 0);
        return std::vector<int>(d->prim_pow + d->ao_prim_off[a], d->prim_pow + d->ao_prim_off[a + 1]);
    };
    auto prim_coefs = [&](int a) { return std::vector<double>(d->prim_coef + d->ao_prim_off[a], d->prim_coef + d->ao_prim_off[a + 1]); };
    for (int a = 0; a < hs.n_ao; ++a) {
        if (used[a]) continue;
        std::vector<double> ex = prim_exps(a);
        std::vector<int> pw = prim_pows(a);
        for (int p : pw) if (p < 0 || p > 6) return QMC_ERR_ARG;
        // find an existing shell with the same key and room
        HostShell* sh = nullptr;
        for (auto& s : hs.shells)
            if (s.nuc == d->ao_nuc[a] && s.exps == ex && s.pows == pw) {
                if (d->ao_l[a] == 0 && (s.s_ao[0] < 0 || s.s_ao[1] < 0)) { sh = &s; break; }
                if (d->ao_l[a] == 1 && s.p_ao[0] < 0) { sh = &s; break; }
            }
        if (!sh) {
            hs.shells.emplace_back();
            sh = &hs.shells.back();
            sh->nuc = d->ao_nuc[a];
            sh->exps = ex;
            sh->pows = pw;
        }
        if (d->ao_l[a] == 0) {
            int slot = sh->s_ao[0] < 0 ? 0 : 1;
            sh->s_ao[slot] = a;
            sh->s_coef[slot] = prim_coefs(a);
            used[a] = 1;
        } else {
            // gather the x, y, z members of this p triplet
            std::vector<double> cf = prim_coefs(a);
            int trip[3] = {-1, -1, -1};
            for (int b = a; b < hs.n_ao; ++b) {
                if (used[b] || d->ao_l[b] != 1 || d->ao_nuc[b] != d->ao_nuc[a]) continue;
                if (prim_exps(b) != ex || prim_coefs(b) != cf) continue;
                int m = d->ao_m[b];
                if (trip[m] < 0) trip[m] = b;
            }
            if (trip[0] < 0 || trip[1] < 0 || trip[2] < 0) return QMC_ERR_ARG;
            for (int m = 0; m < 3; ++m) { sh->p_ao[m] = trip[m]; used[trip[m]] = 1; }
            sh->p_coef = cf;
        }
    }
    std::stable_sort(hs.shells.begin(), hs.shells.end(), [](const HostShell& x, const HostShell& y) { return x.nuc < y.nuc; });
    hs.ao_int.assign(hs.n_ao, -1);
    int nxt = 0;
    for (auto& s : hs.shells) {
        for (int k = 0; k < 2; ++k) if (s.s_ao[k] >= 0) hs.ao_int[s.s_ao[k]] = nxt++;
        if (s.p_ao[0] >= 0) for (int m = 0; m < 3; ++m) hs.ao_int[s.p_ao[m]] = nxt++;
    }
    if (nxt != hs.n_ao) return QMC_ERR_ARG;
    hs.C0.assign(d->mo_coef, d->mo_coef + (size_t)hs.n_mo * hs.n_ao);
    hs.occ.assign(d->occ, d->occ + hs.N);
    for (int e = 0; e < hs.N; ++e) if (hs.occ[e] < 0 || hs.occ[e] >= hs.n_mo) return QMC_ERR_ARG;
    hs.jk = d->jastrow_kind;
    hs.F = d->jas_F;
    if (hs.jk == QMC_JAS_PADE_F && !(hs.F > 0)) return QMC_ERR_ARG;
    for (int i = 0; i < 8; ++i) hs.jas[i] = d->jas[i];
    for (int q = 0; q < d->n_rot; ++q) {
        if (d->rot_occ[q] < 0 || d->rot_occ[q] >= hs.n_mo || d->rot_virt[q] < 0 || d->rot_virt[q] >= hs.n_mo) return QMC_ERR_ARG;
        hs.rot_occ.push_back(d->rot_occ[q]);
        hs.rot_virt.push_back(d->rot_virt[q]);
        hs.rot_angle.push_back(d->rot_angle[q]);
    }
    for (int q = 0; q < d->n_rot; ++q)
        for (int q2 = 0; q2 < q; ++q2) if (hs.rot_occ[q] == hs.rot_occ[q2]) return QMC_ERR_ARG;
    hs.quirks = d->quirks;
    if (d->init_nuc) hs.init_nuc.assign(d->init_nuc, d->init_nuc + hs.N);
    else hs.init_nuc.assign(hs.N, -1);
    for (int e = 0; e < hs.N; ++e) if (hs.init_nuc[e] >= hs.n_nuc) return QMC_ERR_ARG;
    hs.init_sigma = d->init_sigma;
    hs.v_nn = 0.0;
    for (int I = 0; I < hs.n_nuc; ++I)
        for (int J = I + 1; J < hs.n_nuc; ++J) {
            double dx = hs.R[3 * I] - hs.R[3 * J], dy = hs.R[3 * I + 1] - hs.R[3 * J + 1], dz = hs.R[3 * I + 2] - hs.R[3 * J + 2];
            hs.v_nn += hs.Z[I] * hs.Z[J] / std::sqrt(dx * dx + dy * dy + dz * dz);
        }
    // shape
    hs.shape = -1;
    if (hs.N == 2 && hs.n_up == 1 && hs.n_nuc == 2 && hs.basis == QMC_BASIS_STO && hs.jk == QMC_JAS_PADE_F) hs.shape = SHAPE_H2;
    if (hs.N == 3 && hs.n_up == 2 && hs.n_nuc == 1 && hs.basis == QMC_BASIS_STO && hs.jk == QMC_JAS_PADE_F) hs.shape = SHAPE_LI;
    if (hs.N == 10 && hs.n_up == 5 && hs.n_nuc == 5 && hs.basis == QMC_BASIS_GTO && hs.jk == QMC_JAS_PADE_EEN)
        hs.shape = layout_matches_ch4min(hs) ? SHAPE_CH4MIN : SHAPE_CH4;
    if (hs.N == 42 && hs.n_up == 21 && hs.n_nuc == 12 && hs.basis == QMC_BASIS_GTO && hs.jk == QMC_JAS_PADE_EEN &&
        hs.n_ao <= 96)
        hs.shape = SHAPE_C6H6;
    if (hs.shape < 0) return QMC_ERR_UNSUPPORTED;
    return QMC_OK;
}

void free_dev(DevWalkers& dw) {
    cudaFree(dw.pos); cudaFree(dw.dinv); cudaFree(dw.logabs); cudaFree(dw.sign); cudaFree(dw.el);
    cudaFree(dw.flags); cudaFree(dw.acc); cudaFree(dw.partial); cudaFree(dw.rows); cudaFree(dw.chunk_done);
    cudaFree(dw.chunk_jc);
    dw = DevWalkers();
}

int alloc_dev(DevWalkers& dw, const HostSys& hs, int W, int Wcap, int prec, cudaStream_t st) {
    dw.W = W;
    dw.Wcap = ((Wcap + 127) / 128) * 128;
    dw.prec = prec;
    size_t ts = prec == QMC_FP64 ? 8 : 4;
    size_t nd = (size_t)dinv_elems_of_shape(hs.shape);
    size_t Wc = dw.Wcap;
    // block partials of the refresh: up to one block per 4 walkers (warp-per-walker shapes)
    int nblk = (int)((Wc + 3) / 4);
    dw.partial_cap = 2 * nblk + 64;
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess) e = cudaMalloc(&dw.pos, ts * 3 * hs.N * Wc);
    if (e == cudaSuccess) e = cudaMalloc(&dw.dinv, ts * nd * Wc);
    if (e == cudaSuccess) e = cudaMalloc((void**)&dw.logabs, 8 * Wc);
    if (e == cudaSuccess) e = cudaMalloc((void**)&dw.sign, 4 * Wc);
    if (e == cudaSuccess) e = cudaMalloc((void**)&dw.el, 8 * Wc);
    if (e == cudaSuccess) e = cudaMalloc((void**)&dw.flags, 4);
    if (e == cudaSuccess) e = cudaMalloc((void**)&dw.acc, 8);
    if (e == cudaSuccess) e = cudaMalloc((void**)&dw.partial, 8 * (size_t)dw.partial_cap);
    const size_t rb = prec == QMC_FP32_REFINE ? refresh_rows_bytes(hs.shape) : 0;
    if (e == cudaSuccess && rb) e = cudaMalloc((void**)&dw.rows, rb * Wc);
    if (e == cudaSuccess && prec == QMC_FP32_REFINE) e = cudaMalloc((void**)&dw.chunk_done, 4 * (Wc / 32));
    if (e == cudaSuccess) e = cudaMemsetAsync(dw.flags, 0, 4, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(dw.acc, 0, 8, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(dw.sign, 0, 4 * Wc, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(dw.el, 0, 8 * Wc, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(dw.dinv, 0, ts * nd * Wc, st);
    if (e != cudaSuccess) { free_dev(dw); return cuda_rc(e); }
    return QMC_OK;
}

int alloc_walkers(qmc_sys_s* sys, int W, int prec, qmc_walkers_s** out, int capacity = 0) {
    if (W <= 0 || (prec != QMC_FP64 && prec != QMC_FP32_REFINE) || capacity < 0) return QMC_ERR_ARG;
    cudaSetDevice(sys->ctx->device);
    qmc_walkers_s* wk = new (std::nothrow) qmc_walkers_s();
    if (!wk) return QMC_ERR_NOMEM;
    wk->sys = sys;
    const HostSys& hs = sys->hs;
    int cap = std::max(W, capacity);
    int rc = alloc_dev(wk->dw, hs, W, cap, prec, sys->ctx->stream);
    if (rc) { delete wk; return rc; }
    cudaError_t e = cudaMalloc((void**)&wk->d_stage, 8 * 3 * (size_t)hs.N * wk->dw.Wcap);
    if (e != cudaSuccess) { free_dev(wk->dw); delete wk; return cuda_rc(e); }
    *out = wk;
    return QMC_OK;
}

// Lazily allocated DMC buffers: the second population buffer and the
// branching scratch, both of the walker set's capacity.
int ensure_dmc(qmc_walkers_s* wk) {
    if (wk->br.cap) return QMC_OK;
    const HostSys& hs = wk->sys->hs;
    cudaStream_t st = wk->sys->ctx->stream;
    CK(alloc_dev(wk->alt, hs, 0, wk->dw.Wcap, wk->dw.prec, st));
    DevBranch& b = wk->br;
    int cap = wk->dw.Wcap;
    cudaError_t e = cudaMalloc((void**)&b.counts, 4 * (size_t)cap);
    if (e == cudaSuccess) e = cudaMalloc((void**)&b.offsets, 4 * (size_t)cap);
    if (e == cudaSuccess) e = cudaMalloc((void**)&b.el_old, 8 * (size_t)cap);
    if (e == cudaSuccess) e = cudaMalloc((void**)&b.stats, 8 * 4);
    if (e != cudaSuccess) {
        cudaFree(b.counts); cudaFree(b.offsets); cudaFree(b.el_old); cudaFree(b.stats);
        b = DevBranch();
        free_dev(wk->alt);
        return cuda_rc(e);
    }
    b.cap = cap;
    return QMC_OK;
}

void free_walkers(qmc_walkers_s* wk) {
    if (!wk) return;
    free_dev(wk->dw);
    if (wk->br.cap) {
        free_dev(wk->alt);
        cudaFree(wk->br.counts); cudaFree(wk->br.offsets); cudaFree(wk->br.el_old); cudaFree(wk->br.stats);
    }
    cudaFree(wk->d_stage);
    cudaFree(wk->d_out);
    delete wk;
}

int ensure_out(qmc_walkers_s* wk, size_t doubles) {
    if (wk->d_out_cap >= doubles) return QMC_OK;
    cudaFree(wk->d_out);
    wk->d_out = nullptr;
    wk->d_out_cap = 0;
    CU(cudaMalloc((void**)&wk->d_out, doubles * 8));
    wk->d_out_cap = doubles;
    return QMC_OK;
}

// A scratch walker set of at least W walkers for batched evaluation.
int scratch_walkers(qmc_sys_s* sys, int W, int prec, qmc_walkers_s** out) {
    qmc_walkers_s*& s = sys->scratch[prec];
    if (s && s->dw.Wcap >= W) { s->dw.W = W; *out = s; return QMC_OK; }
    free_walkers(s);
    s = nullptr;
    CK(alloc_walkers(sys, W, prec, &s));
    *out = s;
    return QMC_OK;
}

int upload_positions(qmc_walkers_s* wk, const double* pos) {
    const HostSys& hs = wk->sys->hs;
    cudaStream_t st = wk->sys->ctx->stream;
    CU(cudaMemcpyAsync(wk->d_stage, pos, sizeof(double) * 3 * hs.N * (size_t)wk->dw.W, cudaMemcpyHostToDevice, st));
    return launch_scatter_positions(wk->d_stage, wk->dw, wk->sys->d_perm, hs.N, st);
}

// Statistics of a per-step energy series: src/sampling/vmc.rs:141-188.
double autocorrelation_time(const std::vector<double>& x) {
    size_t n = x.size();
    if (n == 0) return 1.0;
    double mean = 0.0;
    for (double v : x) mean += v;
    mean /= (double)n;
    double var = 0.0;
    for (double v : x) var += (v - mean) * (v - mean);
    var /= (double)n;
    if (var == 0.0) return 1.0;
    double tau = 1.0;
    for (size_t t = 1; t < n / 2; ++t) {
        double s = 0.0;
        for (size_t i = 0; i + t < n; ++i) s += (x[i] - mean) * (x[i + t] - mean);
        double a = s / ((double)(n - t) * var);
        if (a < 0.0) break;
        tau += 2.0 * a;
    }
    return tau;
}

double blocking_error(const std::vector<double>& x, double tau) {
    size_t bs = (size_t)std::ceil(2.0 * tau);
    if (bs == 0) bs = 1;
    size_t nb = x.size() / bs;
    if (nb < 2) return 0.0;
    std::vector<double> m(nb, 0.0);
    for (size_t b = 0; b < nb; ++b) {
        for (size_t i = 0; i < bs; ++i) m[b] += x[b * bs + i];
        m[b] /= (double)bs;
    }
    double mu = 0.0;
    for (double v : m) mu += v;
    mu /= (double)nb;
    double var = 0.0;
    for (double v : m) var += (v - mu) * (v - mu);
    var /= (double)(nb - 1);
    return std::sqrt(var / (double)nb);
}

// Blocking error of the DMC energy series (src/sampling/is_dmc.rs:556-607).
double dmc_block_error(const std::vector<double>& x) {
    size_t n = x.size();
    if (n < 20) return 0.0;
    double mean = 0.0;
    for (double v : x) mean += v;
    mean /= (double)n;
    double var = 0.0;
    for (double v : x) var += (v - mean) * (v - mean);
    var /= (double)n;
    if (var < 1e-30) return 0.0;
    double tau = autocorrelation_time(x);
    size_t bs = (size_t)std::ceil(2.0 * tau);
    size_t nb = x.size() / bs;
    if (nb < 2) return std::sqrt(var * tau / (double)n);
    return blocking_error(x, tau);
}

// One IS-DMC step on a resident population: save E_L, one drift-diffusion
// sweep, E_L in the walkers' precision (FP64 when fp64_measure), branching
// and compaction into the alternate buffer, swap.
int dmc_step(qmc_walkers_s* wk, double tau, double tau_move, double max_drift, int fixed_node, double e_ref,
             uint64_t seed, uint64_t step, int fp64_measure, double e_cut, int* n_new, double* e_mean) {
    CK(ensure_dmc(wk));
    const HostSys& hs = wk->sys->hs;
    cudaStream_t st = wk->sys->ctx->stream;
    DevWalkers& dw = wk->dw;
    CU(cudaMemcpyAsync(wk->br.el_old, dw.el, 8 * (size_t)dw.W, cudaMemcpyDeviceToDevice, st));
    dw.fixed_node = fixed_node;
    int rc = launch_sweep(hs, dw, QMC_MOVE_ONE_DRIFT, 1, step, 0.0, tau_move, max_drift, seed, st);
    dw.fixed_node = 0;
    CK(rc);
    MeasureOut none;
    CK(launch_measure(hs, dw, (fp64_measure || dw.prec == QMC_FP64) ? 0 : 1, true, none, st));
    CK(launch_branch(dw, wk->alt, wk->br, hs.N, dinv_elems_of_shape(hs.shape), e_ref, tau, e_cut, seed, step, st));
    double stats[2] = {0, 0};
    CU(cudaMemcpyAsync(stats, wk->br.stats, 16, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    int total = (int)stats[0];
    *n_new = total;
    *e_mean = total > 0 ? stats[1] / total : 0.0;
    if (total > wk->alt.Wcap) return QMC_ERR_POPULATION;
    if (total == 0) { dw.W = 0; return QMC_OK; }
    // swap buffers (flags / accept counters stay with the walker set)
    std::swap(dw.pos, wk->alt.pos);
    std::swap(dw.dinv, wk->alt.dinv);
    std::swap(dw.logabs, wk->alt.logabs);
    std::swap(dw.sign, wk->alt.sign);
    std::swap(dw.el, wk->alt.el);
    dw.W = total;
    return QMC_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// HostSys helpers
// ---------------------------------------------------------------------------
std::vector<double> HostSys::effective_mo() const {
    std::vector<double> C = C0;
    for (size_t q = 0; q < rot_occ.size(); ++q) {
        int k = rot_occ[q], v = rot_virt[q];
        double c = std::cos(rot_angle[q]), s = std::sin(rot_angle[q]);
        for (int a = 0; a < n_ao; ++a) C[(size_t)k * n_ao + a] = c * C0[(size_t)k * n_ao + a] + s * C0[(size_t)v * n_ao + a];
    }
    return C;
}

std::vector<double> HostSys::rotation_derivative_rows() const {
    std::vector<double> D(rot_occ.size() * (size_t)n_ao, 0.0);
    for (size_t q = 0; q < rot_occ.size(); ++q) {
        int k = rot_occ[q], v = rot_virt[q];
        double c = std::cos(rot_angle[q]), s = std::sin(rot_angle[q]);
        for (int a = 0; a < n_ao; ++a) D[q * n_ao + a] = -s * C0[(size_t)k * n_ao + a] + c * C0[(size_t)v * n_ao + a];
    }
    return D;
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

int qmc_version(void) { return 100; }

const char* qmc_status_string(int s) {
    switch (s) {
        case QMC_OK: return "ok";
        case QMC_ERR_ARG: return "invalid argument";
        case QMC_ERR_CUDA: return "CUDA error or no usable device";
        case QMC_ERR_TIMEOUT: return "bounded device wait timed out";
        case QMC_ERR_SINGULAR: return "singular Slater matrix";
        case QMC_ERR_POPULATION: return "DMC population out of range";
        case QMC_ERR_NONFINITE: return "non-finite value";
        case QMC_ERR_UNSUPPORTED: return "no kernel compiled for this system shape";
        case QMC_ERR_NOMEM: return "out of memory";
    }
    return "unknown status";
}

int qmc_init(int device, qmc_ctx_t* out) {
    if (!out) return QMC_ERR_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) { cudaGetLastError(); return QMC_ERR_CUDA; }
    if (device < 0 || device >= n) return QMC_ERR_ARG;
    CU(cudaSetDevice(device));
    qmc_ctx_s* c = new (std::nothrow) qmc_ctx_s();
    if (!c) return QMC_ERR_NOMEM;
    c->device = device;
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    for (int i = 0; i < 16 && e == cudaSuccess; ++i) e = cudaEventCreate(&c->ev[i]);
    if (e != cudaSuccess) { delete c; return cuda_rc(e); }
    c->launches0 = g_launch_count;
    *out = c;
    return QMC_OK;
}

namespace {

// A handle whose owner releases it while children are alive is only marked; the
// memory goes when its last child does. Destruction order between handles is then
// free, as it is for garbage-collected or reference-counted callers.
void free_ctx(qmc_ctx_s* c) {
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    for (int i = 0; i < 16; ++i) if (c->ev[i]) cudaEventDestroy(c->ev[i]);
    if (c->flush_buf) cudaFree(c->flush_buf);
    cudaStreamDestroy(c->stream);
    delete c;
}

void free_sys(qmc_sys_s* s) {
    qmc_ctx_s* c = s->ctx;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    free_walkers(s->scratch[0]);
    free_walkers(s->scratch[1]);
    cudaFree(s->d_perm);
    for (void* t : s->hs.dev_table) cudaFree(t);
    delete s;
    if (--c->n_children == 0 && c->released) free_ctx(c);
}

}  // namespace

int qmc_destroy(qmc_ctx_t c) {
    if (!c || c->released) return QMC_ERR_ARG;
    if (c->n_children > 0) {
        c->released = true;
        return QMC_OK;
    }
    free_ctx(c);
    return QMC_OK;
}

int qmc_system_create(qmc_ctx_t ctx, const qmc_system_desc* desc, qmc_sys_t* out) {
    if (!ctx || !desc || !out || ctx->released) return QMC_ERR_ARG;
    *out = nullptr;
    qmc_sys_s* s = new (std::nothrow) qmc_sys_s();
    if (!s) return QMC_ERR_NOMEM;
    s->ctx = ctx;
    int rc = build_hostsys(desc, s->hs);
    if (rc) { delete s; return rc; }
    cudaSetDevice(ctx->device);
    cudaError_t e = cudaMalloc((void**)&s->d_perm, sizeof(int) * s->hs.N);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(s->d_perm, s->hs.perm.data(), sizeof(int) * s->hs.N, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) { cudaFree(s->d_perm); delete s; return cuda_rc(e); }
    ++ctx->n_children;
    *out = s;
    return QMC_OK;
}

int qmc_system_check(const qmc_system_desc* desc, int* shape) {
    HostSys hs;
    int rc = build_hostsys(desc, hs);
    if (shape) *shape = rc == QMC_OK ? hs.shape : -1;
    return rc;
}

int qmc_roofline_model(const qmc_system_desc* desc, int precision, double acceptance, qmc_roofline_counts* out) {
    if (!desc || !out || (precision != QMC_FP64 && precision != QMC_FP32_REFINE) || !(acceptance >= 0) ||
        acceptance > 1)
        return QMC_ERR_ARG;
    HostSys hs;
    CK(build_hostsys(desc, hs));
    double c[4];
    roofline_counts(hs, precision == QMC_FP64 ? 0 : 1, acceptance, c);
    std::memset(out, 0, sizeof(*out));
    out->sweep_flops_per_move = c[0];
    out->sweep_state_bytes = c[1];
    out->refresh_flops = c[2];
    out->refresh_bytes = c[3];
    return QMC_OK;
}

int qmc_system_destroy(qmc_sys_t s) {
    if (!s || s->released) return QMC_ERR_ARG;
    if (s->n_children > 0) {
        s->released = true;
        return QMC_OK;
    }
    free_sys(s);
    return QMC_OK;
}

int qmc_system_num_params(qmc_sys_t s, int* P) {
    if (!s || !P) return QMC_ERR_ARG;
    *P = s->hs.n_params();
    return QMC_OK;
}

int qmc_system_get_params(qmc_sys_t s, double* p, int P) {
    if (!s || !p || P != s->hs.n_params()) return QMC_ERR_ARG;
    for (int i = 0; i < 8; ++i) p[i] = s->hs.jas[i];
    for (size_t q = 0; q < s->hs.rot_angle.size(); ++q) p[8 + q] = s->hs.rot_angle[q];
    return QMC_OK;
}

int qmc_system_set_params(qmc_sys_t s, const double* p, int P) {
    if (!s || !p || P != s->hs.n_params()) return QMC_ERR_ARG;
    for (int i = 0; i < P; ++i) if (!std::isfinite(p[i])) return QMC_ERR_ARG;
    for (int i = 0; i < 8; ++i) s->hs.jas[i] = p[i];
    for (size_t q = 0; q < s->hs.rot_angle.size(); ++q) s->hs.rot_angle[q] = p[8 + q];
    s->hs.version++;
    return QMC_OK;
}

int qmc_system_set_nuclei(qmc_sys_t s, const double* R, int n_nuc) {
    if (!s || !R || n_nuc != s->hs.n_nuc) return QMC_ERR_ARG;
    for (int i = 0; i < 3 * n_nuc; ++i) if (!std::isfinite(R[i])) return QMC_ERR_ARG;
    s->hs.R.assign(R, R + 3 * n_nuc);
    HostSys& hs = s->hs;
    hs.version++;
    hs.v_nn = 0.0;
    for (int I = 0; I < hs.n_nuc; ++I)
        for (int J = I + 1; J < hs.n_nuc; ++J) {
            double dx = hs.R[3 * I] - hs.R[3 * J], dy = hs.R[3 * I + 1] - hs.R[3 * J + 1], dz = hs.R[3 * I + 2] - hs.R[3 * J + 2];
            hs.v_nn += hs.Z[I] * hs.Z[J] / std::sqrt(dx * dx + dy * dy + dz * dz);
        }
    return QMC_OK;
}

int qmc_eval_batch(qmc_sys_t s, int W, const double* pos, int precision, double* logabs, int* sign,
                   double* grad_ln, double* lap_over_psi, double* e_local) {
    if (!s || W <= 0 || !pos || (precision != QMC_FP64 && precision != QMC_FP32_REFINE)) return QMC_ERR_ARG;
    cudaSetDevice(s->ctx->device);
    cudaStream_t st = s->ctx->stream;
    qmc_walkers_s* wk;
    CK(scratch_walkers(s, W, precision, &wk));
    const HostSys& hs = s->hs;
    int N = hs.N;
    CK(upload_positions(wk, pos));
    CK(ensure_out(wk, (size_t)W * N * 4));
    MeasureOut mo;
    if (grad_ln) mo.grad = wk->d_out;
    if (lap_over_psi) mo.lap = wk->d_out + (size_t)W * N * 3;
    CK(launch_measure(hs, wk->dw, precision == QMC_FP64 ? 0 : 1, true, mo, st));
    std::vector<double> g(grad_ln ? (size_t)W * N * 3 : 0), l(lap_over_psi ? (size_t)W * N : 0);
    if (grad_ln) CU(cudaMemcpyAsync(g.data(), mo.grad, 8 * g.size(), cudaMemcpyDeviceToHost, st));
    if (lap_over_psi) CU(cudaMemcpyAsync(l.data(), mo.lap, 8 * l.size(), cudaMemcpyDeviceToHost, st));
    if (logabs) CU(cudaMemcpyAsync(logabs, wk->dw.logabs, 8 * (size_t)W, cudaMemcpyDeviceToHost, st));
    if (sign) CU(cudaMemcpyAsync(sign, wk->dw.sign, 4 * (size_t)W, cudaMemcpyDeviceToHost, st));
    if (e_local) CU(cudaMemcpyAsync(e_local, wk->dw.el, 8 * (size_t)W, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    for (int w = 0; w < W; ++w)
        for (int ei = 0; ei < N; ++ei) {
            int e = hs.perm[ei];
            if (grad_ln) for (int c = 0; c < 3; ++c) grad_ln[((size_t)w * N + e) * 3 + c] = g[((size_t)w * N + ei) * 3 + c];
            if (lap_over_psi) lap_over_psi[(size_t)w * N + e] = l[(size_t)w * N + ei];
        }
    int fl = 0;
    CU(cudaMemcpy(&fl, wk->dw.flags, 4, cudaMemcpyDeviceToHost));
    CU(cudaMemset(wk->dw.flags, 0, 4));
    return QMC_OK;
}

int qmc_ratio_batch(qmc_sys_t s, int W, const double* pos, int e, const double* r_new, double* ratio,
                    double* grad_ln_new) {
    if (!s || W <= 0 || !pos || !r_new || !ratio || e < 0 || e >= s->hs.N) return QMC_ERR_ARG;
    const int N = s->hs.N;
    std::vector<double> moved(pos, pos + (size_t)W * N * 3);
    for (int w = 0; w < W; ++w)
        for (int c = 0; c < 3; ++c) moved[((size_t)w * N + e) * 3 + c] = r_new[(size_t)w * 3 + c];
    std::vector<double> l0(W), l1(W), g(grad_ln_new ? (size_t)W * N * 3 : 0);
    std::vector<int> s0(W), s1(W);
    CK(qmc_eval_batch(s, W, pos, QMC_FP64, l0.data(), s0.data(), nullptr, nullptr, nullptr));
    CK(qmc_eval_batch(s, W, moved.data(), QMC_FP64, l1.data(), s1.data(), grad_ln_new ? g.data() : nullptr, nullptr,
                      nullptr));
    for (int w = 0; w < W; ++w) {
        ratio[w] = (double)(s0[w] * s1[w]) * std::exp(l1[w] - l0[w]);
        if (grad_ln_new)
            for (int c = 0; c < 3; ++c) grad_ln_new[(size_t)w * 3 + c] = g[((size_t)w * N + e) * 3 + c];
    }
    return QMC_OK;
}

int qmc_logderiv_batch(qmc_sys_t s, int W, const double* pos, double* O, double* e_local, double* dEL, double* S,
                       double* f, double* e_mean) {
    if (!s || W <= 0 || !pos) return QMC_ERR_ARG;
    if (s->hs.jk != QMC_JAS_PADE_EEN) return QMC_ERR_UNSUPPORTED;
    cudaSetDevice(s->ctx->device);
    cudaStream_t st = s->ctx->stream;
    qmc_walkers_s* wk;
    CK(scratch_walkers(s, W, QMC_FP64, &wk));
    const HostSys& hs = s->hs;
    int P = hs.n_params();
    int M = 2 + 2 * P + P * (P + 1) / 2;
    int nblk = std::min(1024, std::max(1, (W + 255) / 256));
    // benzene (OptimizableWfn of BenzeneGTO, src/systems/benzene.rs:726-756):
    // the warp kernels give E_L, a per-walker kernel the Jastrow derivatives;
    // MO-rotation angles would need the determinant and are not compiled
    const bool warp = hs.shape == SHAPE_C6H6;
    if (warp && P != 8) return QMC_ERR_UNSUPPORTED;
    // device scratch: O [W][P], the SR sums and their block partials, the
    // Jastrow table (jas[8], nuclei [n_nuc][5]), then with dEL: dEL [W][P] and
    // grad ln|psi| [W][N][3]
    const size_t base = (size_t)W * P + (size_t)M + 2 * (size_t)M * nblk + 64;
    const size_t ntab = 8 + 5 * (size_t)hs.n_nuc;
    const size_t nd = dEL ? (size_t)W * P + (size_t)W * hs.N * 3 : 0;
    CK(upload_positions(wk, pos));
    CK(ensure_out(wk, base + ntab + nd));
    double* d_tab = wk->d_out + base;
    double* d_dEL = dEL ? d_tab + ntab : nullptr;
    double* d_grad = dEL ? d_dEL + (size_t)W * P : nullptr;
    std::vector<double> tab(hs.jas, hs.jas + 8);
    for (int I = 0; I < hs.n_nuc; ++I) {
        for (int c = 0; c < 3; ++c) tab.push_back(hs.R[3 * I + c]);
        tab.push_back(hs.Z[I]);
        tab.push_back((double)hs.species[I]);
    }
    if (warp || dEL) CU(cudaMemcpyAsync(d_tab, tab.data(), 8 * tab.size(), cudaMemcpyHostToDevice, st));
    MeasureOut mo;
    mo.grad = d_grad;
    if (warp) {
        CK(launch_measure(hs, wk->dw, 0, true, mo, st));          // FP64 refresh: E_L (and grad) on the device
        if (launch_jastrow3_logderiv(wk->dw, hs.N, hs.n_up, hs.n_nuc, d_tab + 8, d_tab, P, wk->d_out, st, d_grad,
                                     d_dEL))
            return QMC_ERR_CUDA;
        mo.O = wk->d_out;
    } else {
        // thread-per-walker shapes: O_p, E_L, grad and the rotation columns of
        // dE_L/dp in one evaluation; the Jastrow columns of dE_L/dp from the
        // gradient afterwards
        mo.O = wk->d_out;
        mo.dEL = d_dEL;
        CK(launch_measure(hs, wk->dw, 0, true, mo, st));
        if (dEL && launch_jastrow3_logderiv(wk->dw, hs.N, hs.n_up, hs.n_nuc, d_tab + 8, d_tab, P, nullptr, st, d_grad,
                                            d_dEL))
            return QMC_ERR_CUDA;
    }
    double* d_sums = wk->d_out + (size_t)W * P;
    double* d_scr = d_sums + M;
    if (S || f || e_mean)
        CK(launch_sr_sums(wk->dw.el, mo.O, W, P, d_sums, d_scr, (int)(2 * (size_t)M * nblk + 64), st));
    if (O) CU(cudaMemcpyAsync(O, mo.O, 8 * (size_t)W * P, cudaMemcpyDeviceToHost, st));
    if (dEL) CU(cudaMemcpyAsync(dEL, d_dEL, 8 * (size_t)W * P, cudaMemcpyDeviceToHost, st));
    if (e_local) CU(cudaMemcpyAsync(e_local, wk->dw.el, 8 * (size_t)W, cudaMemcpyDeviceToHost, st));
    std::vector<double> sums(M);
    if (S || f || e_mean) CU(cudaMemcpyAsync(sums.data(), d_sums, 8 * (size_t)M, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    if (S || f || e_mean) {
        double n = (double)W;
        double Em = sums[0] / n;
        if (e_mean) *e_mean = Em;
        std::vector<double> Om(P);
        for (int p = 0; p < P; ++p) Om[p] = sums[2 + p] / n;
        if (f) for (int p = 0; p < P; ++p) f[p] = sums[2 + P + p] / n - Em * Om[p];
        if (S) {
            int m = 2 + 2 * P;
            for (int p = 0; p < P; ++p)
                for (int q = p; q < P; ++q) {
                    double v = sums[m++] / n - Om[p] * Om[q];
                    S[p * P + q] = v;
                    S[q * P + p] = v;
                }
        }
    }
    return QMC_OK;
}

int qmc_forces_batch(qmc_sys_t s, int W, const double* pos, double* F_hf, double* omega) {
    if (!s || W <= 0 || !pos) return QMC_ERR_ARG;
    cudaSetDevice(s->ctx->device);
    cudaStream_t st = s->ctx->stream;
    qmc_walkers_s* wk;
    CK(scratch_walkers(s, W, QMC_FP64, &wk));
    const HostSys& hs = s->hs;
    size_t per = (size_t)W * hs.n_nuc * 3;
    if (hs.shape == SHAPE_C6H6 || hs.shape == SHAPE_HEG54) {
        // ForceCalculator of BenzeneGTO (src/systems/benzene.rs:811-858):
        // the Hellmann-Feynman force only; wfn_nuclear_gradient is the
        // trait's unimplemented default (src/sampling/traits.rs:50-55).  The
        // electron gas has no nuclei.
        if (omega) return QMC_ERR_UNSUPPORTED;
        if (!F_hf || per == 0) return QMC_OK;
        CK(upload_positions(wk, pos));
        CK(ensure_out(wk, per + 4 * (size_t)hs.n_nuc));
        std::vector<double> nuc(4 * (size_t)hs.n_nuc);
        for (int I = 0; I < hs.n_nuc; ++I) {
            for (int c = 0; c < 3; ++c) nuc[4 * I + c] = hs.R[3 * I + c];
            nuc[4 * I + 3] = hs.Z[I];
        }
        double* d_nuc = wk->d_out + per;
        CU(cudaMemcpyAsync(d_nuc, nuc.data(), 8 * nuc.size(), cudaMemcpyHostToDevice, st));
        if (launch_hf_force_walkers(wk->dw, hs.N, hs.n_nuc, d_nuc, wk->d_out, st)) return QMC_ERR_CUDA;
        CU(cudaMemcpyAsync(F_hf, wk->d_out, 8 * per, cudaMemcpyDeviceToHost, st));
        CU(cudaStreamSynchronize(st));
        return QMC_OK;
    }
    CK(upload_positions(wk, pos));
    CK(ensure_out(wk, 2 * per));
    MeasureOut mo;
    if (F_hf) mo.fhf = wk->d_out;
    if (omega) mo.omega = wk->d_out + per;
    CK(launch_measure(hs, wk->dw, 0, true, mo, st));
    if (F_hf) CU(cudaMemcpyAsync(F_hf, mo.fhf, 8 * per, cudaMemcpyDeviceToHost, st));
    if (omega) CU(cudaMemcpyAsync(omega, mo.omega, 8 * per, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    return QMC_OK;
}

int qmc_walkers_create(qmc_sys_t s, int W, int precision, qmc_walkers_t* out) {
    if (!s || !out || s->released) return QMC_ERR_ARG;
    *out = nullptr;
    CK(alloc_walkers(s, W, precision, out));
    ++s->n_children;
    return QMC_OK;
}

int qmc_walkers_create_dmc(qmc_sys_t s, int W, int capacity, int precision, qmc_walkers_t* out) {
    if (!s || !out || s->released || capacity < W) return QMC_ERR_ARG;
    *out = nullptr;
    CK(alloc_walkers(s, W, precision, out, capacity));
    ++s->n_children;
    return QMC_OK;
}

int qmc_walkers_count(qmc_walkers_t wk, int* W) {
    if (!wk || !W) return QMC_ERR_ARG;
    *W = wk->dw.W;
    return QMC_OK;
}

int qmc_walkers_dmc_step(qmc_walkers_t wk, double tau, double tau_move, double max_drift, int fixed_node,
                         double e_ref, uint64_t seed, uint64_t step, int fp64_measure, double branch_cut, int* n_new,
                         double* e_mean) {
    if (!wk || !n_new || !e_mean || !(tau > 0) || !(tau_move > 0) || !(max_drift > 0) || wk->dw.W <= 0)
        return QMC_ERR_ARG;
    if (!(branch_cut >= 0)) return QMC_ERR_ARG;
    cudaSetDevice(wk->sys->ctx->device);
    return dmc_step(wk, tau, tau_move, max_drift, fixed_node, e_ref, seed, step, fp64_measure, branch_cut, n_new,
                    e_mean);
}

namespace {
void release_walkers(qmc_walkers_s* wk) {
    qmc_sys_s* s = wk->sys;
    cudaSetDevice(s->ctx->device);
    cudaStreamSynchronize(s->ctx->stream);
    free_walkers(wk);
    if (--s->n_children == 0 && s->released) free_sys(s);
}
}  // namespace

int qmc_walkers_destroy(qmc_walkers_t wk) {
    if (!wk || wk->released) return QMC_ERR_ARG;
    if (wk->n_batches > 0) {
        wk->released = true;               // freed when the last batch binding it is destroyed
        return QMC_OK;
    }
    release_walkers(wk);
    return QMC_OK;
}

int qmc_walkers_init(qmc_walkers_t wk, uint64_t seed) {
    if (!wk) return QMC_ERR_ARG;
    cudaSetDevice(wk->sys->ctx->device);
    return launch_init(wk->sys->hs, wk->dw, seed, wk->sys->ctx->stream);
}

int qmc_walkers_set_positions(qmc_walkers_t wk, const double* pos) {
    if (!wk || !pos) return QMC_ERR_ARG;
    cudaSetDevice(wk->sys->ctx->device);
    return upload_positions(wk, pos);
}

int qmc_walkers_get_positions(qmc_walkers_t wk, double* pos) {
    if (!wk || !pos) return QMC_ERR_ARG;
    cudaSetDevice(wk->sys->ctx->device);
    cudaStream_t st = wk->sys->ctx->stream;
    const HostSys& hs = wk->sys->hs;
    CK(launch_gather_positions(wk->dw, wk->d_stage, wk->sys->d_perm, hs.N, st));
    CU(cudaMemcpyAsync(pos, wk->d_stage, sizeof(double) * 3 * hs.N * (size_t)wk->dw.W, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    return QMC_OK;
}

int qmc_walkers_refresh(qmc_walkers_t wk, double* e_local, double* e_sum) {
    if (!wk) return QMC_ERR_ARG;
    cudaSetDevice(wk->sys->ctx->device);
    cudaStream_t st = wk->sys->ctx->stream;
    MeasureOut mo;
    CK(launch_measure(wk->sys->hs, wk->dw, 0, true, mo, st));
    if (e_local) CU(cudaMemcpyAsync(e_local, wk->dw.el, 8 * (size_t)wk->dw.W, cudaMemcpyDeviceToHost, st));
    if (e_sum) CU(cudaMemcpyAsync(e_sum, wk->dw.partial + wk->dw.partial_cap - 1, 8, cudaMemcpyDeviceToHost, st));
    if (e_local || e_sum) CU(cudaStreamSynchronize(st));
    return QMC_OK;
}

int qmc_walkers_rebuild_inverse(qmc_walkers_t wk) {
    if (!wk) return QMC_ERR_ARG;
    cudaSetDevice(wk->sys->ctx->device);
    MeasureOut mo;
    mo.inverse_only = true;
    CK(launch_measure(wk->sys->hs, wk->dw, 0, true, mo, wk->sys->ctx->stream));
    return QMC_OK;
}

int qmc_walkers_sweep(qmc_walkers_t wk, int move_kind, int n_sweeps, uint64_t step0, double step, double tau,
                      double max_drift, uint64_t seed, long long* accepted) {
    if (!wk || n_sweeps < 0 || move_kind < 0 || move_kind > 3) return QMC_ERR_ARG;
    if ((move_kind == QMC_MOVE_ONE_DRIFT) && !(tau > 0 && max_drift > 0)) return QMC_ERR_ARG;
    if (move_kind != QMC_MOVE_ONE_DRIFT && !(step > 0)) return QMC_ERR_ARG;
    if (n_sweeps == 0) { if (accepted) *accepted = 0; return QMC_OK; }
    cudaSetDevice(wk->sys->ctx->device);
    cudaStream_t st = wk->sys->ctx->stream;
    if (accepted) CU(cudaMemsetAsync(wk->dw.acc, 0, 8, st));
    CK(launch_sweep(wk->sys->hs, wk->dw, move_kind, n_sweeps, step0, step, tau, max_drift, seed, st));
    if (accepted) {
        unsigned long long a = 0;
        CU(cudaMemcpyAsync(&a, wk->dw.acc, 8, cudaMemcpyDeviceToHost, st));
        CU(cudaStreamSynchronize(st));
        *accepted = (long long)a;
    }
    return QMC_OK;
}

int qmc_walkers_get_state(qmc_walkers_t wk, double* logabs, int* sign, double* e_local) {
    if (!wk) return QMC_ERR_ARG;
    cudaSetDevice(wk->sys->ctx->device);
    cudaStream_t st = wk->sys->ctx->stream;
    size_t W = wk->dw.W;
    if (logabs) CU(cudaMemcpyAsync(logabs, wk->dw.logabs, 8 * W, cudaMemcpyDeviceToHost, st));
    if (sign) CU(cudaMemcpyAsync(sign, wk->dw.sign, 4 * W, cudaMemcpyDeviceToHost, st));
    if (e_local) CU(cudaMemcpyAsync(e_local, wk->dw.el, 8 * W, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    return QMC_OK;
}

int qmc_walkers_status(qmc_walkers_t wk, int* flags) {
    if (!wk || !flags) return QMC_ERR_ARG;
    cudaSetDevice(wk->sys->ctx->device);
    cudaStream_t st = wk->sys->ctx->stream;
    int f = 0;
    CU(cudaMemcpyAsync(&f, wk->dw.flags, 4, cudaMemcpyDeviceToHost, st));
    CU(cudaMemsetAsync(wk->dw.flags, 0, 4, st));
    CU(cudaStreamSynchronize(st));
    *flags = f;
    return QMC_OK;
}

}  // extern "C"

namespace {

// Step-size / time-step adaptation of the samplers (no device state: the
// rule runs on the host between launches, from the device's acceptance count).
//  MCMCSimulation::adapt_step_size (src/sampling/vmc.rs:122-128):
//    step <- clamp(step * sqrt(rate / target), min, max)
//  DriftDiffusionVMC::adapt_time_step (src/sampling/vmc.rs:397-402):
//    tau <- clamp(tau * clamp(sqrt(rate / target), 0.8, 1.2), 0.001, 0.05)
// applied every adaptation_interval steps (sweeps) over the acceptance of
// that window, through burn-in and production alike (vmc.rs:85-88, 423-428,
// 458-463).  Single-electron Gaussian moves (no reference sampler) adapt their
// width by the MCMC rule.
struct Adapt {
    bool on = false;
    int interval = 0;
    double target = 0.0, lo = 0.0, hi = 0.0;
    bool drift = false;
    unsigned long long acc0 = 0;           // device acceptance count at the window start
    double value = 0.0;                    // current step or tau
    int init(const qmc_run_params* p, bool is_drift, double start) {
        value = start;
        drift = is_drift;
        if (!(p->target_acceptance > 0)) return QMC_OK;
        if (p->target_acceptance >= 1.0 || p->adaptation_interval <= 0) return QMC_ERR_ARG;
        on = true;
        interval = p->adaptation_interval;
        target = p->target_acceptance;
        lo = p->min_step > 0 ? p->min_step : (drift ? 0.001 : 0.0);
        hi = p->max_step > 0 ? p->max_step : (drift ? 0.05 : INFINITY);
        if (!(lo <= hi) || !(value > 0)) return QMC_ERR_ARG;
        return QMC_OK;
    }
    // new window: acceptance count acc after `moves` proposals since acc0
    void update(unsigned long long acc, double moves) {
        const double rate = moves > 0 ? (double)(acc - acc0) / moves : 0.0;
        double f = std::sqrt(rate / target);
        if (drift) f = std::min(1.2, std::max(0.8, f));
        value = std::min(hi, std::max(lo, value * f));
        acc0 = acc;
    }
};

int read_acc(qmc_walkers_s* wk, unsigned long long* acc) {
    cudaStream_t st = wk->sys->ctx->stream;
    CU(cudaMemcpyAsync(acc, wk->dw.acc, 8, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    return QMC_OK;
}

}  // namespace

extern "C" {

int qmc_vmc_run(qmc_sys_t s, const qmc_run_params* p, uint64_t seed, qmc_run_result* res, double* energies) {
    if (!s || !p || !res) return QMC_ERR_ARG;
    if (p->n_walkers <= 0 || p->n_steps <= 0 || p->n_burnin < 0 || p->move_kind < 0 || p->move_kind > 3) return QMC_ERR_ARG;
    std::memset(res, 0, sizeof(*res));
    cudaSetDevice(s->ctx->device);
    cudaStream_t st = s->ctx->stream;
    qmc_walkers_s* wk = nullptr;
    CK(alloc_walkers(s, p->n_walkers, p->precision, &wk));
    struct Guard { qmc_walkers_s* w; ~Guard() { if (w) { cudaStreamSynchronize(w->sys->ctx->stream); free_walkers(w); } } } guard{wk};
    const HostSys& hs = s->hs;
    const bool drift = p->move_kind == QMC_MOVE_ONE_DRIFT;
    Adapt ad;
    CK(ad.init(p, drift, drift ? p->tau : p->step));
    CK(launch_init(hs, wk->dw, seed, st));
    MeasureOut none;
    CK(launch_measure(hs, wk->dw, 0, true, none, st));
    std::vector<double> series;
    long long proposals = 0;
    unsigned long long acc_prod0 = 0;      // acceptance count when production starts
    CU(cudaMemsetAsync(wk->dw.acc, 0, 8, st));
    const double W = (double)wk->dw.W;
    if (p->move_kind == QMC_MOVE_ALL_GAUSS || p->move_kind == QMC_MOVE_ALL_BOX) {
        if (!(p->step > 0)) return QMC_ERR_ARG;
        const int total = p->n_burnin + p->n_steps;
        int nblk = (wk->dw.W + 63) / 64;
        double* d_part = nullptr;
        double* d_mean = nullptr;
        CU(cudaMalloc((void**)&d_part, 16 * (size_t)nblk * p->n_steps));
        cudaError_t e = cudaMalloc((void**)&d_mean, 8 * (size_t)p->n_steps);
        if (e != cudaSuccess) { cudaFree(d_part); return cuda_rc(e); }
        struct Bufs { double* a; double* b; ~Bufs() { cudaFree(a); cudaFree(b); } } bufs{d_part, d_mean};
        // steps t = 0 .. total-1 in launches that end at adaptation points and
        // at the end of the burn-in; production steps record their mean E_L
        int t = 0;
        while (t < total) {
            int end = total;
            if (t < p->n_burnin) end = std::min(end, p->n_burnin);
            if (ad.on) end = std::min(end, (t / ad.interval + 1) * ad.interval);
            const int n = end - t;
            if (t >= p->n_burnin)
                CK(launch_step_all_recorded(hs, wk->dw, p->move_kind, n, (uint64_t)t, ad.value, seed,
                                            d_part + 2 * (size_t)nblk * (t - p->n_burnin), st));
            else
                CK(launch_sweep(hs, wk->dw, p->move_kind, n, (uint64_t)t, ad.value, 0, 0, seed, st));
            t = end;
            if (t == p->n_burnin) CK(read_acc(wk, &acc_prod0));
            if (ad.on && t % ad.interval == 0) {
                unsigned long long acc;
                CK(read_acc(wk, &acc));
                ad.update(acc, (double)ad.interval * W);
            }
        }
        CK(launch_sum_partials(d_part, nblk, p->n_steps, d_mean, st));
        series.resize(p->n_steps);
        CU(cudaMemcpyAsync(series.data(), d_mean, 8 * (size_t)p->n_steps, cudaMemcpyDeviceToHost, st));
        CU(cudaStreamSynchronize(st));
        for (double& v : series) v /= W;
        proposals = (long long)p->n_steps * wk->dw.W;
    } else {
        // single-electron sweeps: the refresh (inverse, log|psi|, E_L) every
        // refresh_every sweeps of the burn-in and of the production, one
        // energy measurement per production refresh; launches also end at
        // adaptation points
        const int every = p->refresh_every > 0 ? p->refresh_every : 1;
        const int total = p->n_burnin + p->n_steps;
        int t = 0, since_refresh = 0;
        while (t < total) {
            int end = total;
            if (t < p->n_burnin) end = std::min(end, p->n_burnin);
            end = std::min(end, t + (every - since_refresh));
            if (ad.on) end = std::min(end, (t / ad.interval + 1) * ad.interval);
            const int n = end - t;
            const double stp = drift ? p->step : ad.value, tau = drift ? ad.value : p->tau;
            CK(launch_sweep(hs, wk->dw, p->move_kind, n, (uint64_t)t, stp, tau, p->max_drift, seed, st));
            if (t >= p->n_burnin) proposals += (long long)n * hs.N * wk->dw.W;
            t = end;
            since_refresh += n;
            const bool burn_end = t == p->n_burnin;
            if (since_refresh == every || burn_end || t == total) {
                CK(launch_measure(hs, wk->dw, 0, true, none, st));
                if (t > p->n_burnin || (t == p->n_burnin && p->n_burnin == 0)) {
                    double esum = 0.0;
                    CU(cudaMemcpyAsync(&esum, wk->dw.partial + wk->dw.partial_cap - 1, 8, cudaMemcpyDeviceToHost, st));
                    CU(cudaStreamSynchronize(st));
                    series.push_back(esum / W);
                }
                since_refresh = 0;
            }
            if (burn_end) CK(read_acc(wk, &acc_prod0));
            if (ad.on && t % ad.interval == 0) {
                unsigned long long acc;
                CK(read_acc(wk, &acc));
                ad.update(acc, (double)ad.interval * hs.N * W);
            }
        }
    }
    res->final_step = ad.value;
    unsigned long long acc = 0;
    int flags = 0;
    CU(cudaMemcpyAsync(&acc, wk->dw.acc, 8, cudaMemcpyDeviceToHost, st));
    CU(cudaMemcpyAsync(&flags, wk->dw.flags, 4, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    double mean = 0.0;
    for (double v : series) mean += v;
    mean /= (double)series.size();
    double var = 0.0;
    for (double v : series) var += (v - mean) * (v - mean);
    res->energy = mean;
    res->variance = series.size() ? var / (double)series.size() : 0.0;
    res->autocorrelation_time = autocorrelation_time(series);
    res->error = blocking_error(series, res->autocorrelation_time);
    res->acceptance_rate = proposals ? (double)(acc - acc_prod0) / (double)proposals : 0.0;
    res->n_samples = (int)series.size();
    res->status_flags = flags;
    if (energies) for (size_t i = 0; i < series.size(); ++i) energies[i] = series[i];
    return QMC_OK;
}

// Device buffers of the Hellmann-Feynman force estimators: nuclei [n_nuc][4],
// block-partial scratch, and one FP64 force sum [3 n_nuc] per recorded step.
struct ForceAcc {
    int n_nuc = 0, n_rows = 0, recorded = 0;
    double* d_nuc = nullptr;
    double* d_partial = nullptr;
    double* d_series = nullptr;
    size_t partial_cap = 0;
    double walkers = 0.0;                  // walker samples summed so far
    ~ForceAcc() { cudaFree(d_nuc); cudaFree(d_partial); cudaFree(d_series); }
    int init(const HostSys& hs, int w_cap, int rows, cudaStream_t st) {
        n_nuc = hs.n_nuc;
        n_rows = rows;
        if (n_nuc == 0) return QMC_OK;
        std::vector<double> nuc(4 * (size_t)n_nuc);
        for (int I = 0; I < n_nuc; ++I) {
            for (int c = 0; c < 3; ++c) nuc[4 * I + c] = hs.R[3 * I + c];
            nuc[4 * I + 3] = hs.Z[I];
        }
        partial_cap = hf_force_scratch_doubles(w_cap, n_nuc);
        CU(cudaMalloc((void**)&d_nuc, 8 * nuc.size()));
        CU(cudaMalloc((void**)&d_partial, 8 * partial_cap));
        CU(cudaMalloc((void**)&d_series, 8 * 3 * (size_t)n_nuc * (rows > 0 ? rows : 1)));
        CU(cudaMemcpyAsync(d_nuc, nuc.data(), 8 * nuc.size(), cudaMemcpyHostToDevice, st));
        return QMC_OK;
    }
    // sum of the electron-nucleus forces of the walker set, one row per call
    int record(const HostSys& hs, const DevWalkers& dw, cudaStream_t st) {
        if (n_nuc == 0) return QMC_OK;
        if (recorded >= n_rows) return QMC_ERR_ARG;
        if (launch_hf_force_sum(dw, hs.N, n_nuc, d_nuc, d_partial, partial_cap, d_series + 3 * (size_t)n_nuc * recorded,
                                st))
            return QMC_ERR_CUDA;
        ++recorded;
        walkers += dw.W;
        return QMC_OK;
    }
    // mean force per walker sample plus the nuclear term of the reference's
    // hellmann_feynman_force (F_I -= sum_J Z_I Z_J (R_I - R_J) / |R_I - R_J|^3)
    int mean(const HostSys& hs, cudaStream_t st, double* out) {
        if (n_nuc == 0) return QMC_OK;
        std::vector<double> rows(3 * (size_t)n_nuc * recorded);
        if (recorded) {
            CU(cudaMemcpyAsync(rows.data(), d_series, 8 * rows.size(), cudaMemcpyDeviceToHost, st));
            CU(cudaStreamSynchronize(st));
        }
        for (int k = 0; k < 3 * n_nuc; ++k) {
            double sum = 0.0, comp = 0.0;               // Neumaier over the recorded steps
            for (int r = 0; r < recorded; ++r) {
                const double v = rows[3 * (size_t)n_nuc * r + k], t = sum + v;
                comp += std::fabs(sum) >= std::fabs(v) ? (sum - t) + v : (v - t) + sum;
                sum = t;
            }
            out[k] = walkers > 0 ? (sum + comp) / walkers : 0.0;
        }
        for (int I = 0; I < n_nuc; ++I)
            for (int J = 0; J < n_nuc; ++J) {
                if (I == J) continue;
                double d[3], r2 = 0.0;
                for (int c = 0; c < 3; ++c) { d[c] = hs.R[3 * I + c] - hs.R[3 * J + c]; r2 += d[c] * d[c]; }
                const double r = std::sqrt(r2);
                if (r > 1e-10)
                    for (int c = 0; c < 3; ++c) out[3 * I + c] -= hs.Z[I] * hs.Z[J] * d[c] / (r2 * r);
            }
        return QMC_OK;
    }
};

// ImportanceSampledDMC::vmc_forces (src/sampling/is_dmc.rs:303-380): min(n_walkers, 50)
// walkers, all-electron Gaussian proposals of width 0.5 (single-electron
// Gaussian sweeps of that width for shapes without an all-electron sampler),
// n_equil steps, then rounds of five steps recording every walker's force
// until n_samples / walkers rounds.
static int vmc_forces(qmc_sys_t s, int n_walkers, int precision, int n_equil, int n_samples, uint64_t seed,
                      double* out) {
    const HostSys& hs = s->hs;
    cudaStream_t st = s->ctx->stream;
    const int W = std::min(n_walkers, 50);
    const int rounds = std::max(1, n_samples / W);
    qmc_walkers_s* wk = nullptr;
    CK(alloc_walkers(s, W, precision, &wk));
    struct Guard { qmc_walkers_s* w; ~Guard() { if (w) { cudaStreamSynchronize(w->sys->ctx->stream); free_walkers(w); } } } guard{wk};
    ForceAcc fa;
    CK(fa.init(hs, W, rounds, st));
    CK(launch_init(hs, wk->dw, seed, st));
    MeasureOut none;
    CK(launch_measure(hs, wk->dw, 0, true, none, st));
    const bool all = hs.shape != SHAPE_C6H6 && hs.shape != SHAPE_HEG54;
    const int mk = all ? QMC_MOVE_ALL_GAUSS : QMC_MOVE_ONE_GAUSS;
    uint64_t step = 0;
    auto advance = [&](int n) -> int {
        if (n <= 0) return QMC_OK;
        CK(launch_sweep(hs, wk->dw, mk, n, step, 0.5, 0.0, 0.0, seed, st));
        step += (uint64_t)n;
        // single-electron sweeps carry FP32 inverses: rebuild them each round
        if (!all) CK(launch_measure(hs, wk->dw, 0, true, none, st));
        return QMC_OK;
    };
    CK(advance(n_equil));
    for (int r = 0; r < rounds; ++r) {
        CK(advance(5));
        CK(fa.record(hs, wk->dw, st));
    }
    return fa.mean(hs, st, out);
}

static int dmc_run_impl(qmc_sys_t s, const qmc_run_params* p, uint64_t seed, qmc_run_result* res, double* energies,
                        double* forces_mixed) {
    if (!s || !p || !res) return QMC_ERR_ARG;
    if (p->n_walkers <= 0 || p->n_steps <= 0 || p->n_burnin < 0 || !(p->tau > 0) || !(p->max_drift > 0)) return QMC_ERR_ARG;
    if (!(p->branch_cut >= 0)) return QMC_ERR_ARG;
    std::memset(res, 0, sizeof(*res));
    cudaSetDevice(s->ctx->device);
    cudaStream_t st = s->ctx->stream;
    const HostSys& hs = s->hs;
    const int target = p->n_walkers;
    qmc_walkers_s* wk = nullptr;
    CK(alloc_walkers(s, target, p->precision, &wk, 4 * target));
    struct Guard { qmc_walkers_s* w; ~Guard() { if (w) { cudaStreamSynchronize(w->sys->ctx->stream); free_walkers(w); } } } guard{wk};
    const double kappa = p->e_ref_damping > 0 ? p->e_ref_damping : 0.5;
    const int every = p->refresh_every > 0 ? p->refresh_every : 1;
    auto reinit = [&](uint64_t key, double& e_ref) -> int {
        wk->dw.W = target;
        CK(launch_init(hs, wk->dw, key, st));
        MeasureOut none;
        CK(launch_measure(hs, wk->dw, 0, true, none, st));
        double esum = 0.0;
        CU(cudaMemcpyAsync(&esum, wk->dw.partial + wk->dw.partial_cap - 1, 8, cudaMemcpyDeviceToHost, st));
        CU(cudaStreamSynchronize(st));
        e_ref = esum / target;                           // initial E_ref = <E_L>, is_dmc.rs:397-398
        return QMC_OK;
    };
    double e_ref = 0.0;
    CK(reinit(seed, e_ref));
    CU(cudaMemsetAsync(wk->dw.acc, 0, 8, st));
    ForceAcc fa;
    if (forces_mixed) CK(fa.init(hs, 4 * target, p->n_steps, st));
    std::vector<double> series;
    double pop_sum = 0.0;
    long long moves = 0;
    unsigned long long acc_burn = 0;
    int collapses = 0;
    const int total_steps = p->n_burnin + p->n_steps;
    for (int t = 0; t < total_steps; ++t) {
        if (t == p->n_burnin) {
            CU(cudaMemcpyAsync(&acc_burn, wk->dw.acc, 8, cudaMemcpyDeviceToHost, st));
            CU(cudaMemsetAsync(wk->dw.acc, 0, 8, st));
        }
        int Wcur = wk->dw.W, n_new = 0;
        double em = 0.0;
        int fp64 = ((t + 1) % every) == 0;
        // The reference diffuses with variance 2 tau and drift 2 tau grad ln psi
        // (is_dmc.rs:218-225) but branches with tau; the Hartree-unit
        // projector needs variance tau and drift tau grad ln psi, i.e. the
        // reference-convention move at tau / 2.
        const double tau_move = p->reference_diffusion ? p->tau : 0.5 * p->tau;
        CK(dmc_step(wk, p->tau, tau_move, p->max_drift, p->fixed_node, e_ref, seed, (uint64_t)t, fp64, p->branch_cut,
                    &n_new, &em));
        if (t >= p->n_burnin) moves += (long long)Wcur * hs.N;
        if (n_new == 0) {                                // collapse: re-initialise, is_dmc.rs:428-437
            ++collapses;
            CK(reinit(seed + 0x9E3779B97F4A7C15ull * (uint64_t)(collapses), e_ref));
            continue;
        }
        if (t >= p->n_burnin) {
            series.push_back(em);
            pop_sum += n_new;
            if (forces_mixed) CK(fa.record(hs, wk->dw, st));   // <F_HF> over the population, is_dmc.rs:479-485
        }
        e_ref = em - kappa * std::log((double)n_new / (double)target) / p->tau;   // is_dmc.rs:489-490
    }
    unsigned long long acc = 0;
    int flags = 0;
    CU(cudaMemcpyAsync(&acc, wk->dw.acc, 8, cudaMemcpyDeviceToHost, st));
    CU(cudaMemcpyAsync(&flags, wk->dw.flags, 4, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    double mean = 0.0;
    for (double v : series) mean += v;
    if (!series.empty()) mean /= (double)series.size();
    double var = 0.0;
    for (double v : series) var += (v - mean) * (v - mean);
    res->energy = mean;
    res->variance = series.empty() ? 0.0 : var / (double)series.size();
    res->autocorrelation_time = autocorrelation_time(series);
    res->error = dmc_block_error(series);
    res->acceptance_rate = moves ? (double)acc / (double)moves : 0.0;
    res->n_samples = (int)series.size();
    res->status_flags = flags | (collapses ? 4 : 0);
    res->avg_population = p->n_steps ? pop_sum / (double)p->n_steps : 0.0;
    if (energies) for (size_t i = 0; i < series.size(); ++i) energies[i] = series[i];
    (void)acc_burn;
    if (forces_mixed) CK(fa.mean(hs, st, forces_mixed));
    return QMC_OK;
}

int qmc_dmc_run(qmc_sys_t s, const qmc_run_params* p, uint64_t seed, qmc_run_result* res, double* energies) {
    return dmc_run_impl(s, p, seed, res, energies, nullptr);
}

int qmc_dmc_run_forces(qmc_sys_t s, const qmc_run_params* p, int n_vmc_equilibrate, int n_vmc_force_samples,
                       uint64_t seed, qmc_run_result* res, double* energies, double* forces_mixed,
                       double* forces_vmc, double* forces_extrapolated) {
    if (!s || !p || !res || !forces_mixed || !forces_vmc || !forces_extrapolated) return QMC_ERR_ARG;
    if (n_vmc_equilibrate < 0 || n_vmc_force_samples < 0 || p->n_walkers <= 0) return QMC_ERR_ARG;
    cudaSetDevice(s->ctx->device);
    const int n3 = 3 * s->hs.n_nuc;
    // Phase 1 of ImportanceSampledDMC::run (is_dmc.rs:388-389), on its own key
    CK(vmc_forces(s, p->n_walkers, p->precision, n_vmc_equilibrate, n_vmc_force_samples,
                  seed ^ 0xD1B54A32D192ED03ull, forces_vmc));
    CK(dmc_run_impl(s, p, seed, res, energies, forces_mixed));
    for (int k = 0; k < n3; ++k) forces_extrapolated[k] = 2.0 * forces_mixed[k] - forces_vmc[k];   // is_dmc.rs:525-530
    return QMC_OK;
}

int qmc_ctx_event_record(qmc_ctx_t c, int slot) {
    if (!c || slot < 0 || slot >= 16) return QMC_ERR_ARG;
    CU(cudaEventRecord(c->ev[slot], c->stream));
    return QMC_OK;
}

int qmc_ctx_event_elapsed(qmc_ctx_t c, int a, int b, float* ms) {
    if (!c || a < 0 || a >= 16 || b < 0 || b >= 16 || !ms) return QMC_ERR_ARG;
    CU(cudaEventSynchronize(c->ev[b]));
    CU(cudaEventElapsedTime(ms, c->ev[a], c->ev[b]));
    return QMC_OK;
}

int qmc_ctx_synchronize(qmc_ctx_t c) {
    if (!c) return QMC_ERR_ARG;
    CU(cudaStreamSynchronize(c->stream));
    return QMC_OK;
}

int qmc_ctx_flush_l2(qmc_ctx_t c) {
    if (!c) return QMC_ERR_ARG;
    cudaSetDevice(c->device);
    if (!c->flush_buf) {
        int l2 = 0;
        cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, c->device);
        c->flush_bytes = std::max<size_t>((size_t)l2 * 2, (size_t)256 << 20);
        CU(cudaMalloc(&c->flush_buf, c->flush_bytes));
    }
    return launch_flush(c->flush_buf, c->flush_bytes, c->stream);
}

int qmc_ctx_launch_count(qmc_ctx_t c, long long* n) {
    if (!c || !n) return QMC_ERR_ARG;
    *n = g_launch_count - c->launches0;
    return QMC_OK;
}

int qmc_ctx_measure_peaks(qmc_ctx_t c, double* fp32_tflops, double* fp64_tflops) {
    if (!c || !fp32_tflops || !fp64_tflops) return QMC_ERR_ARG;
    cudaSetDevice(c->device);
    CK(measure_fma_peak(0, fp32_tflops, c->stream));
    CK(measure_fma_peak(1, fp64_tflops, c->stream));
    return QMC_OK;
}

int qmc_host_alloc(size_t bytes, void** out) {
    if (!out || bytes == 0) return QMC_ERR_ARG;
    CU(cudaMallocHost(out, bytes));
    return QMC_OK;
}

int qmc_host_free(void* p) {
    if (!p) return QMC_ERR_ARG;
    CU(cudaFreeHost(p));
    return QMC_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Uneven batches: many systems advanced together.  Walker sets are grouped
// into classes by (shape, precision); each class launches its sweep and its
// refresh over its (system, walker tile) list: sweeps one block per tile,
// the thread-per-walker refresh as a persistent grid over the tiles.  A step
// (sweeps + FP64 refresh + per-system mean E_L + step-counter advance) is
// captured once into a CUDA graph whose
// class branches run concurrently; the per-call scalars live in a device
// control block, so the same graph replays for every step and every call.
// ---------------------------------------------------------------------------
struct qmc_batch_s {
    struct Cls {
        BatchClass bc;
        std::vector<int> members;          // batch indices, in batch order
        std::vector<BatchRec> recs;
        BatchTile* d_tiles = nullptr;
        BatchRec* d_recs = nullptr;
        int* d_tile_begin = nullptr;
        double* d_partial = nullptr;
        int grid_measure = 0;
        cudaStream_t stream = nullptr;
        cudaEvent_t done = nullptr;
    };
    qmc_ctx_s* ctx = nullptr;
    std::vector<qmc_walkers_s*> wk;
    std::vector<int> versions;             // HostSys::version at the last table upload
    std::vector<Cls> cls;
    BatchCtl* d_ctl = nullptr;
    double* d_series = nullptr;            // [series_rows][n]
    int series_rows = 0;
    cudaEvent_t fork = nullptr;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    bool owns_walkers = false;             // created by qmc_batch_run
};

namespace {

constexpr int kBatchSeriesRows = 1024;

void batch_free(qmc_batch_s* b) {
    if (!b) return;
    cudaSetDevice(b->ctx->device);
    cudaStreamSynchronize(b->ctx->stream);
    for (auto& g : b->graph) if (g) cudaGraphExecDestroy(g);
    for (auto& c : b->cls) {
        if (c.stream) { cudaStreamSynchronize(c.stream); cudaStreamDestroy(c.stream); }
        if (c.done) cudaEventDestroy(c.done);
        cudaFree(c.d_tiles); cudaFree(c.d_recs); cudaFree(c.d_tile_begin); cudaFree(c.d_partial);
    }
    if (b->fork) cudaEventDestroy(b->fork);
    cudaFree(b->d_ctl);
    cudaFree(b->d_series);
    for (qmc_walkers_s* w : b->wk) {
        if (b->owns_walkers) { free_walkers(w); continue; }
        if (--w->n_batches == 0 && w->released) release_walkers(w);
    }
    delete b;
}

// Upload (again) the system tables of every member whose parameters changed.
int batch_sync_tables(qmc_batch_s* b) {
    for (auto& c : b->cls) {
        bool dirty = false;
        for (size_t r = 0; r < c.members.size(); ++r) {
            const int i = c.members[r];
            const HostSys& hs = b->wk[i]->sys->hs;
            if (b->versions[i] == hs.version && c.recs[r].tab_d) continue;
            CK(batch_tables(hs, c.bc.prec, c.recs[r]));
            b->versions[i] = hs.version;
            dirty = true;
        }
        if (dirty) CU(cudaMemcpy(c.d_recs, c.recs.data(), sizeof(BatchRec) * c.recs.size(), cudaMemcpyHostToDevice));
    }
    return QMC_OK;
}

int batch_build(qmc_ctx_s* ctx, const std::vector<qmc_walkers_s*>& wk, bool owns, qmc_batch_s** out) {
    qmc_batch_s* b = new (std::nothrow) qmc_batch_s();
    if (!b) return QMC_ERR_NOMEM;
    b->ctx = ctx;
    b->wk = wk;
    b->owns_walkers = owns;
    b->versions.assign(wk.size(), -1);
    if (!owns) for (qmc_walkers_s* w : wk) ++w->n_batches;
    // on failure the caller keeps the walker sets it passed in
    struct Guard {
        qmc_batch_s* b;
        ~Guard() {
            if (!b) return;
            if (b->owns_walkers) b->wk.clear();
            batch_free(b);
        }
    } guard{b};
    int nsm = 0;
    CU(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device));
    std::map<std::pair<int, int>, int> index;
    for (size_t i = 0; i < wk.size(); ++i) {
        auto key = std::make_pair(wk[i]->sys->hs.shape, wk[i]->dw.prec);
        auto it = index.find(key);
        if (it == index.end()) {
            it = index.emplace(key, (int)b->cls.size()).first;
            b->cls.emplace_back();
            b->cls.back().bc.shape = key.first;
            b->cls.back().bc.prec = key.second;
        }
        b->cls[it->second].members.push_back((int)i);
    }
    for (auto& c : b->cls) {
        const int width = batch_tile_width(c.bc.shape);
        if (width <= 0) return QMC_ERR_UNSUPPORTED;
        std::vector<BatchTile> tiles;
        std::vector<int> begin;
        for (size_t r = 0; r < c.members.size(); ++r) {
            qmc_walkers_s* w = wk[c.members[r]];
            BatchRec rec;
            rec.pos = w->dw.pos;
            rec.dinv = w->dw.dinv;
            rec.sign = w->dw.sign;
            rec.logabs = w->dw.logabs;
            rec.el = w->dw.el;
            rec.acc = w->dw.acc;
            rec.flags = w->dw.flags;
            rec.W = w->dw.W;
            rec.Wcap = w->dw.Wcap;
            rec.index = c.members[r];
            rec.fixed_node = w->dw.fixed_node;
            rec.rows = w->dw.rows;
            if (c.bc.prec == QMC_FP32_REFINE && refresh_rows_bytes(c.bc.shape) && !rec.rows) return QMC_ERR_ARG;
            c.recs.push_back(rec);
            begin.push_back((int)tiles.size());
            for (int w0 = 0; w0 < rec.W; w0 += width) tiles.push_back(BatchTile{(int)r, w0});
        }
        begin.push_back((int)tiles.size());
        c.bc.ntiles = (int)tiles.size();
        c.bc.nrec = (int)c.recs.size();
        CU(cudaMalloc((void**)&c.d_tiles, sizeof(BatchTile) * std::max<size_t>(1, tiles.size())));
        CU(cudaMalloc((void**)&c.d_recs, sizeof(BatchRec) * c.recs.size()));
        CU(cudaMalloc((void**)&c.d_tile_begin, sizeof(int) * begin.size()));
        CU(cudaMalloc((void**)&c.d_partial, 16 * std::max<size_t>(1, tiles.size())));
        if (!tiles.empty())
            CU(cudaMemcpy(c.d_tiles, tiles.data(), sizeof(BatchTile) * tiles.size(), cudaMemcpyHostToDevice));
        CU(cudaMemcpy(c.d_tile_begin, begin.data(), sizeof(int) * begin.size(), cudaMemcpyHostToDevice));
        c.bc.tiles = c.d_tiles;
        c.bc.recs = c.d_recs;
        c.bc.tile_begin = c.d_tile_begin;
        c.bc.tile_partial = c.d_partial;
        // sweeps run one block per tile; the occupancy queries set the kernels'
        // shared-memory attributes before any stream capture
        for (int m = 0; m < 2; ++m) {
            int occ = batch_occupancy(c.bc.shape, c.bc.prec, QMC_MOVE_ONE_GAUSS + m, false);
            if (occ < 0) return -occ;
        }
        // persistent refresh grids of the thread-per-walker shapes: every
        // resident block slot of the GPU (occupancy x SMs)
        int occ = batch_occupancy(c.bc.shape, c.bc.prec, 0, true);
        if (occ < 0) return -occ;
        c.grid_measure = std::max(1, occ) * nsm;
        c.bc.grid_measure = c.grid_measure;
        CU(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
        CU(cudaEventCreateWithFlags(&c.done, cudaEventDisableTiming));
    }
    CU(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
    CU(cudaMalloc((void**)&b->d_ctl, sizeof(BatchCtl)));
    b->series_rows = kBatchSeriesRows;
    CU(cudaMalloc((void**)&b->d_series, 8 * (size_t)b->series_rows * wk.size()));
    CK(batch_sync_tables(b));
    guard.b = nullptr;
    *out = b;
    return QMC_OK;
}

int batch_check_move(const qmc_batch_s* b, int mk) {
    if (mk != QMC_MOVE_ONE_GAUSS && mk != QMC_MOVE_ONE_DRIFT) return QMC_ERR_ARG;
    for (const auto& c : b->cls)
        if (c.bc.shape == SHAPE_HEG54)
            for (const auto& r : c.recs) if (r.fixed_node) return QMC_ERR_UNSUPPORTED;
    return QMC_OK;
}

int batch_upload_ctl(qmc_batch_s* b, const BatchCtl& h) {
    CU(cudaMemcpyAsync(b->d_ctl, &h, sizeof(BatchCtl), cudaMemcpyHostToDevice, b->ctx->stream));
    // pageable source: wait so that `h` may go out of scope
    CU(cudaStreamSynchronize(b->ctx->stream));
    return QMC_OK;
}

// One step on the context stream, class after class (eager form).
int batch_sweep_eager(qmc_batch_s* b, int mk) {
    for (auto& c : b->cls) {
        CK(launch_batch_sweep(c.bc, mk, b->d_ctl, b->ctx->stream));
    }
    return QMC_OK;
}

int batch_measure_eager(qmc_batch_s* b) {
    for (auto& c : b->cls) {
        CK(launch_batch_measure(c.bc, b->ctx->stream));
        CK(launch_batch_energy(c.bc, b->d_ctl, b->d_series, (int)b->wk.size(), b->ctx->stream));
    }
    return QMC_OK;
}

// Capture one step: fork to the class streams, sweep + measure + energy per
// class, join, advance the control block.
int batch_capture(qmc_batch_s* b, int mk, cudaGraphExec_t* out) {
    cudaStream_t st = b->ctx->stream;
    CU(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    int rc = cuda_rc(cudaEventRecord(b->fork, st));
    for (auto& c : b->cls) {
        if (rc) break;
        rc = cuda_rc(cudaStreamWaitEvent(c.stream, b->fork, 0));
        if (!rc) rc = launch_batch_sweep(c.bc, mk, b->d_ctl, c.stream);
        if (!rc) rc = launch_batch_measure(c.bc, c.stream);
        if (!rc) rc = launch_batch_energy(c.bc, b->d_ctl, b->d_series, (int)b->wk.size(), c.stream);
        if (!rc) rc = cuda_rc(cudaEventRecord(c.done, c.stream));
        if (!rc) rc = cuda_rc(cudaStreamWaitEvent(st, c.done, 0));
    }
    if (!rc) rc = launch_batch_advance(b->d_ctl, st);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(st, &g);
    if (!rc && e != cudaSuccess) rc = cuda_rc(e);
    if (!rc) rc = cuda_rc(cudaGraphInstantiate(out, g, 0));
    if (g) cudaGraphDestroy(g);
    return rc;
}

// n_steps graph steps of `sweeps` sweeps each, starting at sweep counter
// step0; series rows (n_steps x n) copied to `series` when given.
int batch_steps(qmc_batch_s* b, int mk, int n_steps, int sweeps, uint64_t step0, double step, double tau,
                double max_drift, uint64_t seed, double* series) {
    CK(batch_check_move(b, mk));
    CK(batch_sync_tables(b));
    cudaGraphExec_t& g = b->graph[mk - QMC_MOVE_ONE_GAUSS];
    if (!g) CK(batch_capture(b, mk, &g));
    cudaStream_t st = b->ctx->stream;
    const size_t n = b->wk.size();
    for (int done = 0; done < n_steps; done += b->series_rows) {
        const int rows = std::min(b->series_rows, n_steps - done);
        BatchCtl h;
        h.step = step0 + (uint64_t)done * (uint64_t)sweeps;
        h.seed = seed;
        h.step_size = step;
        h.tau = tau;
        h.max_drift = max_drift;
        h.n_sweeps = sweeps;
        h.row = 0;
        CK(batch_upload_ctl(b, h));
        for (int r = 0; r < rows; ++r) CU(cudaGraphLaunch(g, st));
        if (series)
            CU(cudaMemcpyAsync(series + (size_t)done * n, b->d_series, 8 * (size_t)rows * n, cudaMemcpyDeviceToHost, st));
        CU(cudaStreamSynchronize(st));
    }
    return QMC_OK;
}

}  // namespace

uint64_t qmc_batch_system_seed(uint64_t seed, int s) { return batch_system_seed(seed, s); }

int qmc_batch_create(qmc_ctx_t ctx, int n, const qmc_walkers_t* walkers, qmc_batch_t* out) {
    if (!ctx || ctx->released || n <= 0 || !walkers || !out) return QMC_ERR_ARG;
    *out = nullptr;
    std::vector<qmc_walkers_s*> wk(walkers, walkers + n);
    for (int i = 0; i < n; ++i) {
        if (!wk[i] || wk[i]->released || wk[i]->sys->ctx != ctx || wk[i]->dw.W <= 0) return QMC_ERR_ARG;
        for (int j = 0; j < i; ++j) if (wk[j] == wk[i]) return QMC_ERR_ARG;
    }
    cudaSetDevice(ctx->device);
    return batch_build(ctx, wk, false, out);
}

int qmc_batch_destroy(qmc_batch_t b) {
    if (!b) return QMC_ERR_ARG;
    batch_free(b);
    return QMC_OK;
}

int qmc_batch_sweep(qmc_batch_t b, int move_kind, int n_sweeps, uint64_t step0, double step, double tau,
                    double max_drift, uint64_t seed) {
    if (!b || n_sweeps < 0) return QMC_ERR_ARG;
    if (move_kind == QMC_MOVE_ONE_DRIFT && !(tau > 0 && max_drift > 0)) return QMC_ERR_ARG;
    if (move_kind == QMC_MOVE_ONE_GAUSS && !(step > 0)) return QMC_ERR_ARG;
    CK(batch_check_move(b, move_kind));
    if (n_sweeps == 0) return QMC_OK;
    cudaSetDevice(b->ctx->device);
    CK(batch_sync_tables(b));
    BatchCtl h;
    h.step = step0;
    h.seed = seed;
    h.step_size = step;
    h.tau = tau;
    h.max_drift = max_drift;
    h.n_sweeps = n_sweeps;
    CK(batch_upload_ctl(b, h));
    CK(batch_sweep_eager(b, move_kind));
    CU(cudaStreamSynchronize(b->ctx->stream));
    return QMC_OK;
}

int qmc_batch_refresh(qmc_batch_t b, double* e_mean) {
    if (!b) return QMC_ERR_ARG;
    cudaSetDevice(b->ctx->device);
    CK(batch_sync_tables(b));
    BatchCtl h;                            // row 0
    CK(batch_upload_ctl(b, h));
    CK(batch_measure_eager(b));
    if (e_mean)
        CU(cudaMemcpyAsync(e_mean, b->d_series, 8 * b->wk.size(), cudaMemcpyDeviceToHost, b->ctx->stream));
    CU(cudaStreamSynchronize(b->ctx->stream));
    return QMC_OK;
}

int qmc_batch_run_steps(qmc_batch_t b, int move_kind, int n_steps, int sweeps_per_step, uint64_t step0, double step,
                        double tau, double max_drift, uint64_t seed, double* e_series) {
    if (!b || n_steps < 0 || sweeps_per_step <= 0) return QMC_ERR_ARG;
    if (move_kind == QMC_MOVE_ONE_DRIFT && !(tau > 0 && max_drift > 0)) return QMC_ERR_ARG;
    if (move_kind == QMC_MOVE_ONE_GAUSS && !(step > 0)) return QMC_ERR_ARG;
    if (n_steps == 0) return QMC_OK;
    cudaSetDevice(b->ctx->device);
    return batch_steps(b, move_kind, n_steps, sweeps_per_step, step0, step, tau, max_drift, seed, e_series);
}

int qmc_batch_run(qmc_ctx_t ctx, int n_sys, const qmc_sys_t* systems, const int* W, const qmc_run_params* p,
                  uint64_t seed, qmc_run_result* per_sys, double* energies) {
    if (!ctx || ctx->released || n_sys <= 0 || !systems || !W || !p || !per_sys) return QMC_ERR_ARG;
    if (p->n_steps <= 0 || p->n_burnin < 0) return QMC_ERR_ARG;
    if (p->move_kind != QMC_MOVE_ONE_GAUSS && p->move_kind != QMC_MOVE_ONE_DRIFT) return QMC_ERR_ARG;
    if (p->move_kind == QMC_MOVE_ONE_DRIFT && !(p->tau > 0 && p->max_drift > 0)) return QMC_ERR_ARG;
    if (p->move_kind == QMC_MOVE_ONE_GAUSS && !(p->step > 0)) return QMC_ERR_ARG;
    if (p->precision != QMC_FP64 && p->precision != QMC_FP32_REFINE) return QMC_ERR_ARG;
    // one captured graph replays a fixed step for every system: no per-system adaptation
    if (p->target_acceptance > 0) return QMC_ERR_UNSUPPORTED;
    for (int i = 0; i < n_sys; ++i)
        if (!systems[i] || systems[i]->released || systems[i]->ctx != ctx || W[i] <= 0) return QMC_ERR_ARG;
    std::memset(per_sys, 0, sizeof(qmc_run_result) * n_sys);
    cudaSetDevice(ctx->device);
    cudaStream_t st = ctx->stream;
    std::vector<qmc_walkers_s*> wk;
    struct WGuard {
        std::vector<qmc_walkers_s*>* v;
        ~WGuard() { if (v) for (auto* w : *v) { cudaStreamSynchronize(w->sys->ctx->stream); free_walkers(w); } }
    } wguard{&wk};
    for (int i = 0; i < n_sys; ++i) {
        qmc_walkers_s* w = nullptr;
        CK(alloc_walkers(systems[i], W[i], p->precision, &w));
        wk.push_back(w);
    }
    // the same start as qmc_vmc_run of each system with its batch seed
    MeasureOut none;
    for (int i = 0; i < n_sys; ++i) {
        CK(launch_init(systems[i]->hs, wk[i]->dw, batch_system_seed(seed, i), st));
        CK(launch_measure(systems[i]->hs, wk[i]->dw, 0, true, none, st));
    }
    qmc_batch_s* b = nullptr;
    CK(batch_build(ctx, wk, true, &b));
    wguard.v = nullptr;                    // the batch frees the walker sets
    struct BGuard { qmc_batch_s* b; ~BGuard() { batch_free(b); } } bguard{b};
    const int every = p->refresh_every > 0 ? p->refresh_every : 1;
    const int mk = p->move_kind;
    // burn-in: full steps, then the remainder
    const int nb_full = p->n_burnin / every, nb_rem = p->n_burnin % every;
    uint64_t sweep = 0;
    if (nb_full) CK(batch_steps(b, mk, nb_full, every, sweep, p->step, p->tau, p->max_drift, seed, nullptr));
    sweep += (uint64_t)nb_full * every;
    if (nb_rem) CK(batch_steps(b, mk, 1, nb_rem, sweep, p->step, p->tau, p->max_drift, seed, nullptr));
    sweep += (uint64_t)nb_rem;
    for (qmc_walkers_s* w : wk) CU(cudaMemsetAsync(w->dw.acc, 0, 8, st));
    const int ns_full = p->n_steps / every, ns_rem = p->n_steps % every;
    const int rows = ns_full + (ns_rem ? 1 : 0);
    std::vector<double> series((size_t)rows * n_sys);
    if (ns_full) CK(batch_steps(b, mk, ns_full, every, sweep, p->step, p->tau, p->max_drift, seed, series.data()));
    sweep += (uint64_t)ns_full * every;
    if (ns_rem)
        CK(batch_steps(b, mk, 1, ns_rem, sweep, p->step, p->tau, p->max_drift, seed,
                       series.data() + (size_t)ns_full * n_sys));
    for (int i = 0; i < n_sys; ++i) {
        unsigned long long acc = 0;
        int flags = 0;
        CU(cudaMemcpyAsync(&acc, wk[i]->dw.acc, 8, cudaMemcpyDeviceToHost, st));
        CU(cudaMemcpyAsync(&flags, wk[i]->dw.flags, 4, cudaMemcpyDeviceToHost, st));
        CU(cudaStreamSynchronize(st));
        std::vector<double> e(rows);
        for (int r = 0; r < rows; ++r) e[r] = series[(size_t)r * n_sys + i];
        double mean = 0.0;
        for (double v : e) mean += v;
        mean /= (double)rows;
        double var = 0.0;
        for (double v : e) var += (v - mean) * (v - mean);
        qmc_run_result& res = per_sys[i];
        res.energy = mean;
        res.variance = var / (double)rows;
        res.autocorrelation_time = autocorrelation_time(e);
        res.error = blocking_error(e, res.autocorrelation_time);
        const double proposals = (double)p->n_steps * systems[i]->hs.N * W[i];
        res.acceptance_rate = (double)acc / proposals;
        res.n_samples = rows;
        res.status_flags = flags;
    }
    if (energies) std::memcpy(energies, series.data(), sizeof(double) * series.size());
    return QMC_OK;
}

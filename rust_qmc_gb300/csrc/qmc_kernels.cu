// qmc_kernels.cu -- shape-independent kernels (walker reductions, L2
// flush, position scatter/gather) and the dispatch from a system's shape to
// the per-shape kernel instantiations in qmc_shape_*.cu.
#include <cstdio>
#include <cstring>
#include <algorithm>
#include "qmc_internal.h"
#include "qmc_device.cuh"
#include "qmc_jastrow3_logderiv.h"

namespace qmc {

long long g_launch_count = 0;

static int cuda_status(cudaError_t e) {
    if (e != cudaSuccess) {
        std::fprintf(stderr, "qmc_gb300: CUDA error %s\n", cudaGetErrorString(e));
        return 2;
    }
    return 0;
}

#define QMC_DECLARE_SHAPE(NAME)                                                                               \
    int shape_init_##NAME(const HostSys&, DevWalkers&, uint64_t, cudaStream_t);                              \
    int shape_measure_##NAME(const HostSys&, DevWalkers&, int, bool, const MeasureOut&, cudaStream_t);       \
    int shape_sweep_one_##NAME(const HostSys&, DevWalkers&, int, int, uint64_t, double, double, double,      \
                               uint64_t, cudaStream_t);                                                      \
    int shape_step_all_##NAME(const HostSys&, DevWalkers&, int, int, uint64_t, double, uint64_t, cudaStream_t,\
                              double*);                                                                      \
    int shape_nmax_##NAME();
#define QMC_DECLARE_BATCH(NAME)                                                                               \
    int shape_batch_sweep_##NAME(const BatchClass&, int, const BatchCtl*, cudaStream_t, int*);                \
    int shape_batch_measure_##NAME(const BatchClass&, cudaStream_t, int*);                                    \
    int shape_batch_tables_##NAME(const HostSys&, int, BatchRec&);                                            \
    int shape_batch_width_##NAME();
QMC_DECLARE_BATCH(h2)
QMC_DECLARE_BATCH(li)
QMC_DECLARE_BATCH(ch4)
QMC_DECLARE_BATCH(ch4min)
QMC_DECLARE_BATCH(c6h6)
QMC_DECLARE_BATCH(heg)
QMC_DECLARE_SHAPE(h2)
QMC_DECLARE_SHAPE(li)
QMC_DECLARE_SHAPE(ch4)
QMC_DECLARE_SHAPE(ch4min)
QMC_DECLARE_SHAPE(c6h6)
QMC_DECLARE_SHAPE(heg)

size_t refresh_rows_bytes(int shape) {
    // N electrons x (5 NMAX + 7) float-float quantities (see RowLayout)
    auto b = [](int ne, int nm) { return (size_t)8 * ne * (5 * nm + 7); };
    switch (shape) {
        case SHAPE_H2: return b(ShapeH2::NE, ShapeH2::NMAX);
        case SHAPE_LI: return b(ShapeLi::NE, ShapeLi::NMAX);
        case SHAPE_CH4: return b(ShapeCH4::NE, ShapeCH4::NMAX);
        case SHAPE_CH4MIN: return b(ShapeCH4Min::NE, ShapeCH4Min::NMAX);
        // two-pass electron-gas refresh: 7 float-float terms per electron (54)
        case SHAPE_HEG54: return (size_t)8 * 54 * 7;
    }
    return 0;
}

int dinv_elems_of_shape(int shape) {
    int nm = nmax_of_shape(shape);
    return 2 * nm * nm * (shape == SHAPE_HEG54 ? 2 : 1);
}

// The compile-time CH4 layout has no all-electron kernels of its own.
int shape_step_all_ch4min(const HostSys& hs, DevWalkers& dw, int mk, int n, uint64_t s0, double step, uint64_t seed,
                          cudaStream_t st, double* partial) {
    return shape_step_all_ch4(hs, dw, mk, n, s0, step, seed, st, partial);
}

bool layout_matches_ch4min(const HostSys& hs) {
    using LY = LayoutCH4Min;
    if ((int)hs.shells.size() != LY::NSHELL || hs.n_ao != 9) return false;
    for (int s = 0; s < LY::NSHELL; ++s) {
        const HostShell& h = hs.shells[s];
        if (h.nuc != LY::nuc(s) || (int)h.exps.size() != LY::np(s)) return false;
        bool has_p = h.p_ao[0] >= 0;
        if (h.s_ao[0] < 0 || h.s_ao[1] >= 0 || has_p != (LY::kind(s) == 2)) return false;
    }
    return true;
}

#define QMC_SHAPE_SWITCH(shape, CALL)                  \
    switch (shape) {                                   \
        case SHAPE_H2: return CALL(h2);                \
        case SHAPE_LI: return CALL(li);                \
        case SHAPE_CH4: return CALL(ch4);              \
        case SHAPE_CH4MIN: return CALL(ch4min);        \
        case SHAPE_C6H6: return CALL(c6h6);            \
        case SHAPE_HEG54: return CALL(heg);            \
    }                                                  \
    return 7;

int nmax_of_shape(int shape) {
#define C_(n) shape_nmax_##n()
    QMC_SHAPE_SWITCH(shape, C_)
#undef C_
}

int launch_init(const HostSys& hs, DevWalkers& dw, uint64_t seed, cudaStream_t st) {
#define C_(n) shape_init_##n(hs, dw, seed, st)
    QMC_SHAPE_SWITCH(hs.shape, C_)
#undef C_
}

int launch_measure(const HostSys& hs, DevWalkers& dw, int compute_prec, bool write_state, const MeasureOut& out,
                   cudaStream_t st) {
#define C_(n) shape_measure_##n(hs, dw, compute_prec, write_state, out, st)
    QMC_SHAPE_SWITCH(hs.shape, C_)
#undef C_
}

int launch_sweep(const HostSys& hs, DevWalkers& dw, int move_kind, int n_sweeps, uint64_t step0, double step,
                 double tau, double max_drift, uint64_t seed, cudaStream_t st) {
    if (move_kind == 0 || move_kind == 1) {
        if (hs.shape == SHAPE_CH4MIN) return shape_step_all_ch4(hs, dw, move_kind, n_sweeps, step0, step, seed, st, nullptr);
#define C_(n) shape_step_all_##n(hs, dw, move_kind, n_sweeps, step0, step, seed, st, nullptr)
        QMC_SHAPE_SWITCH(hs.shape, C_)
#undef C_
    }
#define C_(n) shape_sweep_one_##n(hs, dw, move_kind, n_sweeps, step0, step, tau, max_drift, seed, st)
    QMC_SHAPE_SWITCH(hs.shape, C_)
#undef C_
}

// All-electron steps with per-step E_L partial sums recorded.
int launch_step_all_recorded(const HostSys& hs, DevWalkers& dw, int move_kind, int n, uint64_t s0, double step,
                             uint64_t seed, double* partial, cudaStream_t st) {
    if (move_kind != 0 && move_kind != 1) return 1;
    if (hs.shape == SHAPE_CH4MIN) return shape_step_all_ch4(hs, dw, move_kind, n, s0, step, seed, st, partial);
#define C_(nm) shape_step_all_##nm(hs, dw, move_kind, n, s0, step, seed, st, partial)
    QMC_SHAPE_SWITCH(hs.shape, C_)
#undef C_
}

// Final reduction of block partial pairs: out[j] = sum over blocks of
// partial[j][b] (pairs (s,c)).  One block per row: a fixed-order strided pass over the row's compensated
// block partials, then a fixed-order tree (deterministic for a given nblk).
__global__ void __launch_bounds__(256) k_sum_partials(const double* __restrict__ partial, int nblk, int nrows,
                                                      double* __restrict__ out) {
    const int j = blockIdx.x, t = threadIdx.x;
    if (j >= nrows) return;
    __shared__ double ss[256], sc[256];
    Comp acc{0.0, 0.0};
    const double* p = partial + (size_t)j * 2 * nblk;
    for (int b = t; b < nblk; b += 256) {
        acc = comp_add(acc, Comp{p[2 * b], 0.0});
        acc.c += p[2 * b + 1];
    }
    ss[t] = acc.s;
    sc[t] = acc.c;
    __syncthreads();
#pragma unroll
    for (int o = 128; o > 0; o >>= 1) {
        if (t < o) {
            Comp c = comp_add(Comp{ss[t], sc[t]}, Comp{ss[t + o], sc[t + o]});
            ss[t] = c.s;
            sc[t] = c.c;
        }
        __syncthreads();
    }
    if (t == 0) out[j] = ss[0] + sc[0];
}

// SR sums: quantity m over the walkers of chunk b, Neumaier-compensated,
// fixed order.  Quantities: 0 E, 1 E^2, 2..2+P-1 O_p, 2+P..2+2P-1 E O_p,
// then O_p O_q for p <= q (row-major upper triangle).
__device__ __forceinline__ double sr_quantity(int m, int P, const double* E, const double* O, int w) {
    double e = E[w];
    if (m == 0) return e;
    if (m == 1) return e * e;
    if (m < 2 + P) return O[(size_t)w * P + (m - 2)];
    if (m < 2 + 2 * P) return e * O[(size_t)w * P + (m - 2 - P)];
    int k = m - 2 - 2 * P;
    int p = 0;
    while (k >= P - p) { k -= P - p; ++p; }
    int q = p + k;
    return O[(size_t)w * P + p] * O[(size_t)w * P + q];
}

__global__ void k_sr_partials(const double* __restrict__ E, const double* __restrict__ O, int W, int P, int M,
                              int chunk, double* __restrict__ partial, int nblk) {
    int m = threadIdx.x;
    int b = blockIdx.x;
    if (m >= M) return;
    int w0 = b * chunk, w1 = min(W, w0 + chunk);
    Comp acc{0.0, 0.0};
    for (int w = w0; w < w1; ++w) acc = comp_add(acc, Comp{sr_quantity(m, P, E, O, w), 0.0});
    partial[((size_t)m * nblk + b) * 2] = acc.s;
    partial[((size_t)m * nblk + b) * 2 + 1] = acc.c;
}

__global__ void k_flush(uint4* buf, size_t n, unsigned v) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (; i < n; i += stride) buf[i] = make_uint4(v, v + 1, v + 2, v + 3);
}

int launch_sr_sums(const double* E, const double* O, int W, int P, double* d_out, double* d_scratch,
                   int scratch_cap, cudaStream_t st) {
    int M = 2 + 2 * P + P * (P + 1) / 2;
    int nblk = std::min(1024, std::max(1, (W + 255) / 256));
    int chunk = (W + nblk - 1) / nblk;
    nblk = (W + chunk - 1) / chunk;
    if ((size_t)2 * M * nblk > (size_t)scratch_cap) return 8;
    int tpb = ((M + 31) / 32) * 32;
    if (tpb > 1024) return 1;
    k_sr_partials<<<nblk, tpb, 0, st>>>(E, O, W, P, M, chunk, d_scratch, nblk);
    ++g_launch_count;
    k_sum_partials<<<M, 256, 0, st>>>(d_scratch, nblk, M, d_out);
    ++g_launch_count;
    return cuda_status(cudaGetLastError());
}

int launch_walker_sum(const double* X, int W, int ncol, double* d_out, double* d_scratch, int scratch_cap,
                      cudaStream_t st) {
    (void)ncol;
    return launch_sr_sums(X, X, W, 0, d_out, d_scratch, scratch_cap, st);
}

// Hellmann-Feynman electron-nucleus forces summed over walkers
// (src/systems/methane.rs:1247-1256, hydrogen.rs:233-243, benzene.rs:834-844):
// walker w contributes f_I = Z_I sum_i (r_i - R_I) / |r_i - R_I|^3, pairs
// closer than 1e-10 skipped.  One compensated partial per block and force
// component, partial[3 I + c][block]; nuc = [n_nuc][4] (x, y, z, Z).
template <class TS, int TPB>
__global__ void __launch_bounds__(TPB) k_hf_force_partials(const TS* __restrict__ pos, int W, int Wcap, int N,
                                                           int n_nuc, const double* __restrict__ nuc,
                                                           double* __restrict__ partial, int nblk) {
    const int w = blockIdx.x * TPB + threadIdx.x;
    const bool act = w < W;
    for (int I = 0; I < n_nuc; ++I) {
        const double X = nuc[4 * I], Y = nuc[4 * I + 1], Zc = nuc[4 * I + 2], Q = nuc[4 * I + 3];
        double fx = 0.0, fy = 0.0, fz = 0.0;
        if (act) {
            for (int i = 0; i < N; ++i) {
                const double dx = (double)pos[(size_t)(3 * i) * Wcap + w] - X;
                const double dy = (double)pos[(size_t)(3 * i + 1) * Wcap + w] - Y;
                const double dz = (double)pos[(size_t)(3 * i + 2) * Wcap + w] - Zc;
                const double d2 = dx * dx + dy * dy + dz * dz;
                const double d = sqrt(d2);
                if (d > 1e-10) {
                    const double f = Q / (d2 * d);
                    fx += f * dx; fy += f * dy; fz += f * dz;
                }
            }
        }
        block_partial<TPB>(fx, partial + (size_t)(3 * I + 0) * 2 * nblk, blockIdx.x);
        block_partial<TPB>(fy, partial + (size_t)(3 * I + 1) * 2 * nblk, blockIdx.x);
        block_partial<TPB>(fz, partial + (size_t)(3 * I + 2) * 2 * nblk, blockIdx.x);
    }
}

// Per-walker Hellmann-Feynman force for the shapes whose evaluation kernels
// carry no force outputs (src/systems/benzene.rs:828-858, the form of
// methane.rs:1241-1272): F[w][I] = Z_I sum_i (r_i - R_I) / |r_i - R_I|^3
// - sum_{J != I} Z_I Z_J (R_I - R_J) / |R_I - R_J|^3, distances below 1e-10
// skipped.  One thread per (walker, nucleus), t = w n_nuc + I, which is also
// the output row; nuc = [n_nuc][4] (x, y, z, Z).
template <class TS>
__global__ void k_hf_force_walkers(const TS* __restrict__ pos, int W, int Wcap, int N, int n_nuc,
                                   const double* __restrict__ nuc, double* __restrict__ F) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= W * n_nuc) return;
    const int w = t / n_nuc, I = t - w * n_nuc;
    const double X = nuc[4 * I], Y = nuc[4 * I + 1], Zc = nuc[4 * I + 2], Q = nuc[4 * I + 3];
    double fx = 0.0, fy = 0.0, fz = 0.0;
    for (int i = 0; i < N; ++i) {
        const double dx = (double)pos[(size_t)(3 * i) * Wcap + w] - X;
        const double dy = (double)pos[(size_t)(3 * i + 1) * Wcap + w] - Y;
        const double dz = (double)pos[(size_t)(3 * i + 2) * Wcap + w] - Zc;
        const double d2 = dx * dx + dy * dy + dz * dz;
        const double d = sqrt(d2);
        if (d > 1e-10) {
            const double f = Q / (d2 * d);
            fx += f * dx; fy += f * dy; fz += f * dz;
        }
    }
    for (int J = 0; J < n_nuc; ++J) {
        if (J == I) continue;
        const double dx = X - nuc[4 * J], dy = Y - nuc[4 * J + 1], dz = Zc - nuc[4 * J + 2];
        const double d2 = dx * dx + dy * dy + dz * dz;
        const double d = sqrt(d2);
        if (d > 1e-10) {
            const double f = Q * nuc[4 * J + 3] / (d2 * d);
            fx -= f * dx; fy -= f * dy; fz -= f * dz;
        }
    }
    F[(size_t)t * 3] = fx;
    F[(size_t)t * 3 + 1] = fy;
    F[(size_t)t * 3 + 2] = fz;
}

int launch_hf_force_walkers(const DevWalkers& dw, int N, int n_nuc, const double* d_nuc, double* d_out,
                            cudaStream_t st) {
    const long long n = (long long)dw.W * n_nuc;
    if (n <= 0) return 0;
    if (n > 0x7fffffffLL) return 1;
    const int tpb = 128;
    const int nb = (int)((n + tpb - 1) / tpb);
    if (dw.prec == 0)
        k_hf_force_walkers<double><<<nb, tpb, 0, st>>>((const double*)dw.pos, dw.W, dw.Wcap, N, n_nuc, d_nuc, d_out);
    else
        k_hf_force_walkers<float><<<nb, tpb, 0, st>>>((const float*)dw.pos, dw.W, dw.Wcap, N, n_nuc, d_nuc, d_out);
    ++g_launch_count;
    return cuda_status(cudaGetLastError());
}

// Jastrow3 parameter log-derivatives, one thread per walker, for the shapes
// whose evaluation kernels carry no O_p outputs (qmc_jastrow3_logderiv.h):
// O[w][0..7] with row stride P (skipped when O is null); par = p[8],
// nuc = [n_nuc][5] (x, y, z, Z, species 0 or 1: the host rejects other
// species when it builds a system).  With grad ([W][N][3], grad_i ln|psi| in
// the internal electron order) the Jastrow-parameter derivatives of the
// local energy go to dEL[w][0..7], same stride.
template <class TS>
__global__ void k_jastrow3_logderiv(const TS* __restrict__ pos, int W, int Wcap, int N, int n_up, int n_nuc,
                                    const double* __restrict__ nuc, const double* __restrict__ par, int P,
                                    double* __restrict__ O, const double* __restrict__ grad,
                                    double* __restrict__ dEL) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= W) return;
    auto at = [&](int i, int c) { return (double)pos[(size_t)(3 * i + c) * Wcap + w]; };
    double o[8];
    if (O) {
        jastrow3_log_derivatives(N, n_up, n_nuc, nuc, par, at, o);
#pragma unroll
        for (int k = 0; k < 8; ++k) O[(size_t)w * P + k] = o[k];
    }
    if (grad && dEL) {
        const double* g = grad + (size_t)w * N * 3;
        auto gr = [&](int i, int c) { return g[3 * i + c]; };
        jastrow3_el_derivatives(N, n_up, n_nuc, nuc, par, at, gr, o);
#pragma unroll
        for (int k = 0; k < 8; ++k) dEL[(size_t)w * P + k] = o[k];
    }
}

int launch_jastrow3_logderiv(const DevWalkers& dw, int N, int n_up, int n_nuc, const double* d_nuc,
                             const double* d_par, int P, double* d_O, cudaStream_t st, const double* d_grad,
                             double* d_dEL) {
    if (dw.W <= 0) return 0;
    if (P < 8) return 1;
    const int tpb = 128;
    const int nb = (dw.W + tpb - 1) / tpb;
    if (dw.prec == 0)
        k_jastrow3_logderiv<double><<<nb, tpb, 0, st>>>((const double*)dw.pos, dw.W, dw.Wcap, N, n_up, n_nuc, d_nuc,
                                                        d_par, P, d_O, d_grad, d_dEL);
    else
        k_jastrow3_logderiv<float><<<nb, tpb, 0, st>>>((const float*)dw.pos, dw.W, dw.Wcap, N, n_up, n_nuc, d_nuc,
                                                       d_par, P, d_O, d_grad, d_dEL);
    ++g_launch_count;
    return cuda_status(cudaGetLastError());
}

size_t hf_force_scratch_doubles(int W, int n_nuc) { return (size_t)2 * ((W + 127) / 128) * 3 * n_nuc; }

int launch_hf_force_sum(const DevWalkers& dw, int N, int n_nuc, const double* d_nuc, double* d_partial,
                        size_t partial_cap, double* d_out, cudaStream_t st) {
    constexpr int TPB = 128;
    if (n_nuc <= 0 || dw.W <= 0) return 0;
    const int nblk = (dw.W + TPB - 1) / TPB;
    if (hf_force_scratch_doubles(dw.W, n_nuc) > partial_cap) return 1;
    if (dw.prec == 0)
        k_hf_force_partials<double, TPB><<<nblk, TPB, 0, st>>>((const double*)dw.pos, dw.W, dw.Wcap, N, n_nuc, d_nuc,
                                                               d_partial, nblk);
    else
        k_hf_force_partials<float, TPB><<<nblk, TPB, 0, st>>>((const float*)dw.pos, dw.W, dw.Wcap, N, n_nuc, d_nuc,
                                                              d_partial, nblk);
    ++g_launch_count;
    int rc = cuda_status(cudaGetLastError());
    if (rc) return rc;
    return launch_sum_partials(d_partial, nblk, 3 * n_nuc, d_out, st);
}

int launch_flush(void* buf, size_t bytes, cudaStream_t st) {
    size_t n = bytes / sizeof(uint4);
    k_flush<<<152 * 8, 256, 0, st>>>((uint4*)buf, n, (unsigned)(g_launch_count & 0xffff));
    ++g_launch_count;
    return cuda_status(cudaGetLastError());
}

template <class TS>
__global__ void k_scatter(const double* __restrict__ src, TS* __restrict__ pos, const int* __restrict__ perm, int N,
                          int W, int Wcap) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N * W) return;
    int ei = i / W, w = i - ei * W;
    int e = perm[ei];
#pragma unroll
    for (int c = 0; c < 3; ++c) pos[(size_t)(3 * ei + c) * Wcap + w] = (TS)src[((size_t)w * N + e) * 3 + c];
}

template <class TS>
__global__ void k_gather(const TS* __restrict__ pos, double* __restrict__ dst, const int* __restrict__ perm, int N,
                         int W, int Wcap) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N * W) return;
    int ei = i / W, w = i - ei * W;
    int e = perm[ei];
#pragma unroll
    for (int c = 0; c < 3; ++c) dst[((size_t)w * N + e) * 3 + c] = (double)pos[(size_t)(3 * ei + c) * Wcap + w];
}

int launch_scatter_positions(const double* src, DevWalkers& dw, const int* d_perm, int N, cudaStream_t st) {
    int n = N * dw.W, tpb = 256;
    if (dw.prec == 0) k_scatter<double><<<(n + tpb - 1) / tpb, tpb, 0, st>>>(src, (double*)dw.pos, d_perm, N, dw.W, dw.Wcap);
    else k_scatter<float><<<(n + tpb - 1) / tpb, tpb, 0, st>>>(src, (float*)dw.pos, d_perm, N, dw.W, dw.Wcap);
    ++g_launch_count;
    return cuda_status(cudaGetLastError());
}

int launch_gather_positions(const DevWalkers& dw, double* dst, const int* d_perm, int N, cudaStream_t st) {
    int n = N * dw.W, tpb = 256;
    if (dw.prec == 0) k_gather<double><<<(n + tpb - 1) / tpb, tpb, 0, st>>>((const double*)dw.pos, dst, d_perm, N, dw.W, dw.Wcap);
    else k_gather<float><<<(n + tpb - 1) / tpb, tpb, 0, st>>>((const float*)dw.pos, dst, d_perm, N, dw.W, dw.Wcap);
    ++g_launch_count;
    return cuda_status(cudaGetLastError());
}

// ---------------------------------------------------------------------------
// Uneven batches: dispatch by shape class, per-system energies, step counter.
// ---------------------------------------------------------------------------
int batch_tile_width(int shape) {
#define C_(n) shape_batch_width_##n()
    QMC_SHAPE_SWITCH(shape, C_)
#undef C_
}

int batch_tables(const HostSys& hs, int prec, BatchRec& rec) {
#define C_(n) shape_batch_tables_##n(hs, prec, rec)
    QMC_SHAPE_SWITCH(hs.shape, C_)
#undef C_
}

int launch_batch_sweep(const BatchClass& bc, int move_kind, const BatchCtl* ctl, cudaStream_t st) {
#define C_(n) shape_batch_sweep_##n(bc, move_kind, ctl, st, nullptr)
    QMC_SHAPE_SWITCH(bc.shape, C_)
#undef C_
}

int launch_batch_measure(const BatchClass& bc, cudaStream_t st) {
#define C_(n) shape_batch_measure_##n(bc, st, nullptr)
    QMC_SHAPE_SWITCH(bc.shape, C_)
#undef C_
}

int batch_occupancy(int shape, int prec, int move_kind, bool measure) {
    BatchClass bc;
    bc.shape = shape;
    bc.prec = prec;
    int occ = 0, rc = 7;
#define C_(n) (measure ? shape_batch_measure_##n(bc, nullptr, &occ) : shape_batch_sweep_##n(bc, move_kind, nullptr, nullptr, &occ))
    switch (shape) {
        case SHAPE_H2: rc = C_(h2); break;
        case SHAPE_LI: rc = C_(li); break;
        case SHAPE_CH4: rc = C_(ch4); break;
        case SHAPE_CH4MIN: rc = C_(ch4min); break;
        case SHAPE_C6H6: rc = C_(c6h6); break;
        case SHAPE_HEG54: rc = C_(heg); break;
    }
#undef C_
    return rc ? -rc : occ;
}

// One warp per system: the system's tile partials (contiguous, fixed order)
// summed with compensation, divided by its walker count.
__global__ void k_batch_energy(const BatchRec* __restrict__ recs, int nrec, const int* __restrict__ tile_begin,
                               const double* __restrict__ tile_partial, const BatchCtl* __restrict__ ctl,
                               double* __restrict__ series, int n_total) {
    const int r = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (r >= nrec) return;
    Comp c{0.0, 0.0};
    for (int t = tile_begin[r] + lane; t < tile_begin[r + 1]; t += 32)
        c = comp_add(c, Comp{tile_partial[2 * t], tile_partial[2 * t + 1]});
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        Comp d{__shfl_down_sync(0xffffffffu, c.s, o), __shfl_down_sync(0xffffffffu, c.c, o)};
        c = comp_add(c, d);
    }
    if (lane == 0) {
        const BatchRec& R = recs[r];
        series[(size_t)ctl->row * n_total + R.index] = (c.s + c.c) / (double)R.W;
    }
}

int launch_batch_energy(const BatchClass& bc, const BatchCtl* ctl, double* series, int n_total, cudaStream_t st) {
    if (bc.nrec == 0) return 0;
    const int wpb = 4;
    k_batch_energy<<<(bc.nrec + wpb - 1) / wpb, 32 * wpb, 0, st>>>(bc.recs, bc.nrec, bc.tile_begin, bc.tile_partial,
                                                                   ctl, series, n_total);
    ++g_launch_count;
    return cuda_status(cudaGetLastError());
}

__global__ void k_batch_advance(BatchCtl* ctl) {
    ctl->step += (unsigned long long)ctl->n_sweeps;
    ctl->row += 1;
}

int launch_batch_advance(BatchCtl* ctl, cudaStream_t st) {
    k_batch_advance<<<1, 1, 0, st>>>(ctl);
    ++g_launch_count;
    return cuda_status(cudaGetLastError());
}

int launch_sum_partials(const double* partial, int nblk, int nrows, double* out, cudaStream_t st) {
    k_sum_partials<<<nrows, 256, 0, st>>>(partial, nblk, nrows, out);
    ++g_launch_count;
    return cuda_status(cudaGetLastError());
}


// ---------------------------------------------------------------------------
// DMC branching (src/sampling/is_dmc.rs:278-302) with on-device compaction.
// ---------------------------------------------------------------------------
// Copies per walker: m = min(floor(exp(tau (E_ref - (E_L + E_old)/2)) + xi), 3),
// FP64 log-weight, xi from the tag-4 Philox draw of (walker slot, step).
// Walkers with a non-finite energy get no copy.
__global__ void k_branch_counts(const double* __restrict__ el, const double* __restrict__ el_old, int W,
                                double e_ref, double tau, double e_cut, uint64_t seed, uint64_t step,
                                int* __restrict__ counts, int* flags) {
    int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= W) return;
    double e = el[w], eo = el_old[w];
    int m = 0;
    if (isfinite(e) && isfinite(eo)) {
        double eb = 0.5 * (e + eo);
        if (e_cut > 0.0) eb = fmin(e_ref + e_cut, fmax(e_ref - e_cut, eb));
        double logw = tau * (e_ref - eb);
        U4 x = rng_draw(seed, (uint32_t)w, step, 0, TAG_BRANCH);
        double f = floor(exp(logw) + to_u01(x.x, 0.0));
        m = f >= 3.0 ? 3 : (f <= 0.0 ? 0 : (int)f);
    } else {
        atomicOr(flags, FLAG_NONFINITE);
    }
    counts[w] = m;
}

// One block: exclusive scan of the counts (offsets), the new population size
// and the compensated sum of copies x E_L, in a fixed order.
__global__ void __launch_bounds__(1024) k_branch_scan(const int* __restrict__ counts, const double* __restrict__ el,
                                                      int W, int* __restrict__ offsets, double* __restrict__ stats) {
    __shared__ int ssum[1024];
    __shared__ double se[1024], sc[1024];
    const int t = threadIdx.x;
    const int per = (W + 1023) / 1024;
    const int b = min(W, t * per), e = min(W, b + per);
    int local = 0;
    Comp ce{0.0, 0.0};
    for (int i = b; i < e; ++i) {
        int c = counts[i];
        local += c;
        if (c) ce = comp_add(ce, Comp{(double)c * el[i], 0.0});
    }
    ssum[t] = local;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        int v = t >= off ? ssum[t - off] : 0;
        __syncthreads();
        ssum[t] += v;
        __syncthreads();
    }
    int run = ssum[t] - local;
    for (int i = b; i < e; ++i) { offsets[i] = run; run += counts[i]; }
    se[t] = ce.s;
    sc[t] = ce.c;
    __syncthreads();
    for (int o = 512; o > 0; o >>= 1) {
        if (t < o) {
            Comp x = comp_add(Comp{se[t], sc[t]}, Comp{se[t + o], sc[t + o]});
            se[t] = x.s;
            sc[t] = x.c;
        }
        __syncthreads();
    }
    if (t == 0) {
        stats[0] = (double)ssum[1023];
        stats[1] = se[0] + sc[0];
    }
}

// Order-stable gather: destination slot d takes the walker w with
// offsets[w] <= d < offsets[w] + counts[w] (the last w with offsets[w] <= d).
template <class TS>
__global__ void k_branch_gather(const int* __restrict__ offsets, int W, const double* __restrict__ stats, int cap,
                                const TS* __restrict__ spos, const TS* __restrict__ sdinv,
                                const double* __restrict__ slog, const int* __restrict__ ssign,
                                const double* __restrict__ sel, int sWcap, TS* __restrict__ dpos,
                                TS* __restrict__ ddinv, double* __restrict__ dlog, int* __restrict__ dsign,
                                double* __restrict__ del, int dWcap, int npos, int ndinv) {
    int d = blockIdx.x * blockDim.x + threadIdx.x;
    int total = (int)stats[0];
    if (d >= total || d >= cap) return;
    int lo = 0, hi = W - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (offsets[mid] <= d) lo = mid; else hi = mid - 1;
    }
    const int w = lo;
    for (int i = 0; i < npos; ++i) dpos[(size_t)i * dWcap + d] = spos[(size_t)i * sWcap + w];
    for (int i = 0; i < ndinv; ++i) ddinv[(size_t)i * dWcap + d] = sdinv[(size_t)i * sWcap + w];
    dlog[d] = slog[w];
    dsign[d] = ssign[w];
    del[d] = sel[w];
}

int launch_branch(DevWalkers& src, DevWalkers& dst, DevBranch& br, int n_elec, int nmax, double e_ref, double tau,
                  double e_cut, uint64_t seed, uint64_t step, cudaStream_t st) {
    int W = src.W;
    if (W <= 0 || W > br.cap) return 1;
    k_branch_counts<<<(W + 255) / 256, 256, 0, st>>>(src.el, br.el_old, W, e_ref, tau, e_cut, seed, step,
                                                       br.counts, src.flags);
    k_branch_scan<<<1, 1024, 0, st>>>(br.counts, src.el, W, br.offsets, br.stats);
    int most = std::min(3 * W, dst.Wcap);
    int npos = 3 * n_elec, ndinv = nmax;   // caller passes the per-walker inverse-block size
    if (src.prec == 0)
        k_branch_gather<double><<<(most + 127) / 128, 128, 0, st>>>(
            br.offsets, W, br.stats, dst.Wcap, (const double*)src.pos, (const double*)src.dinv, src.logabs,
            src.sign, src.el, src.Wcap, (double*)dst.pos, (double*)dst.dinv, dst.logabs, dst.sign, dst.el, dst.Wcap,
            npos, ndinv);
    else
        k_branch_gather<float><<<(most + 127) / 128, 128, 0, st>>>(
            br.offsets, W, br.stats, dst.Wcap, (const float*)src.pos, (const float*)src.dinv, src.logabs,
            src.sign, src.el, src.Wcap, (float*)dst.pos, (float*)dst.dinv, dst.logabs, dst.sign, dst.el, dst.Wcap,
            npos, ndinv);
    g_launch_count += 3;
    return cuda_status(cudaGetLastError());
}

// FMA-chain kernels used to measure the SIMT peaks (roofline denominators for
// the compute-bound sweep kernels).  8 independent chains per thread.
template <class T>
__global__ void k_fma_peak(T* out, int iters, T a, T b) {
    T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 16; ++u) {
            x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
            x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
        }
    }
    T s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == T(-1.2345)) out[0] = s;
}

int measure_fma_peak(int fp64, double* tflops, cudaStream_t st) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    void* out = nullptr;
    if (cudaMalloc(&out, 16) != cudaSuccess) return 8;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    int blocks = sms * 8, tpb = 256, iters = fp64 ? 64 : 2048;
    float ms = 0.f;
    for (int rep = 0; rep < 2; ++rep) {
        cudaEventRecord(a, st);
        if (fp64) k_fma_peak<double><<<blocks, tpb, 0, st>>>((double*)out, iters, 0.999999, 1e-7);
        else k_fma_peak<float><<<blocks, tpb, 0, st>>>((float*)out, iters, 0.999999f, 1e-7f);
        cudaEventRecord(b, st);
        cudaEventSynchronize(b);
        cudaEventElapsedTime(&ms, a, b);
    }
    g_launch_count += 2;
    int rc = cuda_status(cudaGetLastError());
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(out);
    double flops = 2.0 * 8 * 16 * (double)iters * blocks * tpb;
    *tflops = ms > 0 ? flops / (ms * 1e-3) / 1e12 : 0.0;
    return rc;
}

}  // namespace qmc

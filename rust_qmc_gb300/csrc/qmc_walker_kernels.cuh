// qmc_walker_kernels.cuh -- templated CUDA kernels of the walker path
// (sm_103a), instantiated once per system shape in qmc_shape_*.cu.
//
//   k_init       MultiWfn::initialize for every walker (Philox, tag 3)
//   k_measure    full evaluation from positions: AO->MO, Gauss-Jordan inverse
//                and log-determinant, Jastrow, grad/Laplacian, E_L, optional
//                parameter log-derivatives and nuclear forces.  In FP64 it is
//                the refresh of the FP32 walkers (inverse + E_L every N sweeps)
//   k_sweep_one  single-electron Metropolis / Langevin sweeps with
//                Sherman-Morrison inverse updates, n sweeps per launch, walker
//                state resident in shared memory for the whole launch
//   k_step_all   all-electron Metropolis steps (H2 path of MCMCSimulation)
#pragma once
#include <cstdio>
#include <cstring>
#include <cmath>
#include <vector>
#include <algorithm>
#include <utility>
#include "qmc_internal.h"
#include "qmc_device.cuh"

namespace qmc {


// ---------------------------------------------------------------------------
// Host: fill the device table of a shape from the host description.
// ---------------------------------------------------------------------------
template <class SH, class T>
static bool fill_sys(const HostSys& hs, SysT<SH, T>& S) {
    std::memset(&S, 0, sizeof(S));
    if (hs.N != SH::NE || hs.n_up != SH::NUP || hs.n_nuc != SH::NNUC) return false;
    if ((int)hs.shells.size() > SH::NSH || hs.n_ao > SH::NAO || (int)hs.rot_occ.size() > SH::NROT) return false;
    for (int I = 0; I < SH::NNUC; ++I) {
        for (int c = 0; c < 3; ++c) S.nuc[I][c] = (T)hs.R[3 * I + c];
        S.Z[I] = (T)hs.Z[I];
        int sp = hs.species[I];
        S.species[I] = sp;
        S.Aspec[I] = (T)hs.jas[6 + sp];
        S.enA[I] = (T)(hs.jas[6 + sp] * hs.Z[I]);
        S.enB[I] = (T)hs.jas[4 + sp];
    }
    S.F = (T)hs.F;
    S.invF = (T)(1.0 / hs.F);
    S.b_ee[0] = (T)hs.jas[0]; S.b_ee[1] = (T)hs.jas[1];
    S.a_ee[0] = (T)hs.jas[2]; S.a_ee[1] = (T)hs.jas[3];
    S.qa = (hs.quirks & 1) ? (T)hs.F : (T)1;
    S.quirk_lap = (hs.quirks & 2) ? 1 : 0;
    S.v_nn = (T)hs.v_nn;
    S.n_rot = (int)hs.rot_occ.size();
    // shells (already sorted by nucleus)
    int np = 0;
    for (int I = 0; I <= SH::NNUC; ++I) S.sh_start[I] = 0;
    for (size_t s = 0; s < hs.shells.size(); ++s) {
        const HostShell& h = hs.shells[s];
        S.sh_start[h.nuc + 1]++;
        if (np + (int)h.exps.size() > SH::NPRIM) return false;
        S.sh_p0[s] = np;
        S.sh_np[s] = (int)h.exps.size();
        S.sh_s0[s] = h.s_ao[0] >= 0 ? hs.ao_int[h.s_ao[0]] : -1;
        S.sh_s1[s] = h.s_ao[1] >= 0 ? hs.ao_int[h.s_ao[1]] : -1;
        S.sh_p[s] = h.p_ao[0] >= 0 ? hs.ao_int[h.p_ao[0]] : -1;
        for (size_t p = 0; p < h.exps.size(); ++p) {
            S.pexp[np] = (T)h.exps[p];
            S.pexp2[np] = (T)(-h.exps[p] * 1.4426950408889634);
            S.ppow[np] = h.pows.empty() ? 0 : h.pows[p];
            S.cs0[np] = h.s_ao[0] >= 0 ? (T)h.s_coef[0][p] : (T)0;
            S.cs1[np] = h.s_ao[1] >= 0 ? (T)h.s_coef[1][p] : (T)0;
            S.cp[np] = h.p_ao[0] >= 0 ? (T)h.p_coef[p] : (T)0;
            ++np;
        }
    }
    for (int I = 0; I < SH::NNUC; ++I) S.sh_start[I + 1] += S.sh_start[I];
    // MO columns per sector, internal AO order
    std::vector<double> Ce = hs.effective_mo();
    for (int sig = 0; sig < 2; ++sig) {
        int col = 0;
        for (int ei = 0; ei < hs.N; ++ei) {
            int e = hs.perm[ei];
            if ((hs.spins[e] > 0) != (sig == 0)) continue;
            int k = hs.occ[e];
            for (int a = 0; a < hs.n_ao; ++a) S.C[sig][hs.ao_int[a]][col] = (T)Ce[(size_t)k * hs.n_ao + a];
            ++col;
        }
    }
    std::vector<double> dC = hs.rotation_derivative_rows();
    for (size_t q = 0; q < hs.rot_occ.size(); ++q) {
        for (int a = 0; a < hs.n_ao; ++a) S.dC[q][hs.ao_int[a]] = (T)dC[q * hs.n_ao + a];
        for (int sig = 0; sig < 2; ++sig) {
            S.rot_col[q][sig] = -1;
            int col = 0;
            for (int ei = 0; ei < hs.N; ++ei) {
                int e = hs.perm[ei];
                if ((hs.spins[e] > 0) != (sig == 0)) continue;
                if (hs.occ[e] == hs.rot_occ[q]) S.rot_col[q][sig] = col;
                ++col;
            }
        }
    }
    S.init_sigma = (T)hs.init_sigma;
    for (int ei = 0; ei < hs.N; ++ei) {
        S.perm[ei] = hs.perm[ei];
        S.init_nuc[ei] = hs.init_nuc[hs.perm[ei]];
    }
    return true;
}

// ---------------------------------------------------------------------------
// Jastrow sums for one electron e against all others (+ nuclei): u and,
// with GRAD, grad_e u.  `pos(j, c)` returns coordinate c of electron j.
// ---------------------------------------------------------------------------
template <class SH, class T, int SIG, bool GRAD, class PosFn>
__device__ __forceinline__ T jastrow_point(const SysT<SH, T>& S, PosFn pos, int e, T x, T y, T z,
                                           T& gx, T& gy, T& gz) {
    T u = 0;
    gx = 0; gy = 0; gz = 0;
    if (SH::JAS == JAS_NONE) return u;
#pragma unroll
    for (int j = 0; j < SH::NE; ++j) {
        if (j == e) continue;
        const bool para = ((j < SH::NUP) == (SIG == 0));
        T dx = x - pos(j, 0), dy = y - pos(j, 1), dz = z - pos(j, 2);
        T d, ri;
        dist(dx * dx + dy * dy + dz * dz, d, ri);
        T uu, upr, lt;
        if (SH::JAS == JAS_PADE_F) pade_f(S.F, S.invF, d, ri, uu, upr, lt);
        else pade_ab(S.a_ee[para ? 1 : 0], S.b_ee[para ? 1 : 0], d, ri, uu, upr, lt);
        u += uu;
        if (GRAD) { gx += upr * dx; gy += upr * dy; gz += upr * dz; }
    }
    if (SH::JAS == JAS_PADE_EEN) {
#pragma unroll
        for (int I = 0; I < SH::NNUC; ++I) {
            T dx = x - S.nuc[I][0], dy = y - S.nuc[I][1], dz = z - S.nuc[I][2];
            T d, ri;
            dist(dx * dx + dy * dy + dz * dz, d, ri);
            T uu, upr, lt;
            pade_ab(S.enA[I], S.enB[I], d, ri, uu, upr, lt);
            u -= uu;
            if (GRAD) { gx -= upr * dx; gy -= upr * dy; gz -= upr * dz; }
        }
    }
    if (GRAD) { gx *= S.qa; gy *= S.qa; gz *= S.qa; }
    return u;
}

// Change of u when electron e moves from (ox,oy,oz) to (nx,ny,nz): old and
// new pair terms in one branch-free pass (the partner e itself is masked),
// optionally with grad_e u at both positions.
template <class SH, class T, int SIG, bool GRAD, class PosFn>
__device__ __forceinline__ T jastrow_delta(const SysT<SH, T>& S, PosFn pos, int e, T ox, T oy, T oz, T nx, T ny,
                                           T nz, T (&go)[3], T (&gn)[3]) {
    T du = 0;
    go[0] = go[1] = go[2] = gn[0] = gn[1] = gn[2] = 0;
    if (SH::JAS == JAS_NONE) return du;
#pragma unroll
    for (int j = 0; j < SH::NE; ++j) {
        const bool para = ((j < SH::NUP) == (SIG == 0));
        const T m = (j != e) ? T(1) : T(0);
        T xj = pos(j, 0), yj = pos(j, 1), zj = pos(j, 2);
        T ax = ox - xj, ay = oy - yj, az = oz - zj;
        T bx = nx - xj, by = ny - yj, bz = nz - zj;
        T ra = ax * ax + ay * ay + az * az, rb = bx * bx + by * by + bz * bz;
        ra = (j != e) ? ra : T(1);
        rb = (j != e) ? rb : T(1);
        T da, ia, db, ib;
        dist(ra, da, ia);
        dist(rb, db, ib);
        T ua, upa, lta, ub, upb, ltb;
        if (SH::JAS == JAS_PADE_F) {
            pade_f(S.F, S.invF, da, ia, ua, upa, lta);
            pade_f(S.F, S.invF, db, ib, ub, upb, ltb);
        } else {
            const int c = para ? 1 : 0;
            pade_ab(S.a_ee[c], S.b_ee[c], da, ia, ua, upa, lta);
            pade_ab(S.a_ee[c], S.b_ee[c], db, ib, ub, upb, ltb);
        }
        du += m * (ub - ua);
        if (GRAD) {
            upa *= m; upb *= m;
            go[0] += upa * ax; go[1] += upa * ay; go[2] += upa * az;
            gn[0] += upb * bx; gn[1] += upb * by; gn[2] += upb * bz;
        }
    }
    if (SH::JAS == JAS_PADE_EEN) {
#pragma unroll
        for (int I = 0; I < SH::NNUC; ++I) {
            T ax = ox - S.nuc[I][0], ay = oy - S.nuc[I][1], az = oz - S.nuc[I][2];
            T bx = nx - S.nuc[I][0], by = ny - S.nuc[I][1], bz = nz - S.nuc[I][2];
            T da, ia, db, ib;
            dist(ax * ax + ay * ay + az * az, da, ia);
            dist(bx * bx + by * by + bz * bz, db, ib);
            T ua, upa, lta, ub, upb, ltb;
            pade_ab(S.enA[I], S.enB[I], da, ia, ua, upa, lta);
            pade_ab(S.enA[I], S.enB[I], db, ib, ub, upb, ltb);
            du -= ub - ua;
            if (GRAD) {
                go[0] -= upa * ax; go[1] -= upa * ay; go[2] -= upa * az;
                gn[0] -= upb * bx; gn[1] -= upb * by; gn[2] -= upb * bz;
            }
        }
    }
    if (GRAD) {
#pragma unroll
        for (int c = 0; c < 3; ++c) { go[c] *= S.qa; gn[c] *= S.qa; }
    }
    return du;
}

// ---------------------------------------------------------------------------
// Electron-pair cache of the Gaussian single-electron sweep.  The sweep keeps
// u(r_ij) of every pair i > j in shared memory (slot i (i - 1) / 2 + j), so a
// proposal evaluates only the new pair terms of the moving electron; the old
// ones are the cached values, which are bit-identical to a recomputation
// (same expression on the same squared distance).  One extra slot, held at
// zero, is the in-bounds target of the masked self pair.
// ---------------------------------------------------------------------------
template <class SH, int MOVE>
__host__ __device__ constexpr int sweep_pairs() {
    return (MOVE == MOVE_ONE_GAUSS && SH::JAS != JAS_NONE) ? SH::NE * (SH::NE - 1) / 2 + 1 : 0;
}
// Shared-memory words per walker of the single-electron sweep: positions,
// the two inverse Slater matrices, the pair cache.
template <class SH, int MOVE>
__host__ __device__ constexpr int sweep_words() {
    return 3 * SH::NE + 2 * SH::NMAX * SH::NMAX + sweep_pairs<SH, MOVE>();
}

template <class T>
__device__ __forceinline__ T sq3(T x, T y, T z) { return x * x + y * y + z * z; }

// 1/r from r^2; +inf at r = 0, so that a / (b + 1/r) gives the r -> 0 limit 0.
__device__ __forceinline__ float inv_r(float r2) { return rsqrtf(r2); }
__device__ __forceinline__ double inv_r(double r2) { return r2 > 0.0 ? frsqrt(r2) : (double)INFINITY; }

// Pade a r / (1 + b r) evaluated as a / (b + 1/r).
template <class T>
__device__ __forceinline__ T pade_value(T a, T b, T r2) { return a * frcp(b + inv_r(r2)); }

// Electron-electron u of one pair at squared distance r2.
template <class SH, class T>
__device__ __forceinline__ T pair_u(const SysT<SH, T>& S, bool para, T r2) {
    if (SH::JAS == JAS_PADE_F) {
        T d, ri, u, up, lt;
        dist(r2, d, ri);
        pade_f(S.F, S.invF, d, ri, u, up, lt);
        return u;
    }
    return pade_value(S.a_ee[para ? 1 : 0], S.b_ee[para ? 1 : 0], r2);
}

// Fill the pair cache pc (this thread's column, stride TPB) from positions.
template <class SH, class T, int TPB, class PosFn>
__device__ __forceinline__ void pair_cache_fill(const SysT<SH, T>& S, PosFn pos, T* pc) {
#pragma unroll 1
    for (int i = 1; i < SH::NE; ++i) {
#pragma unroll 1
        for (int j = 0; j < i; ++j) {
            const bool para = (i < SH::NUP) == (j < SH::NUP);
            T r2 = sq3(pos(i, 0) - pos(j, 0), pos(i, 1) - pos(j, 1), pos(i, 2) - pos(j, 2));
            pc[(i * (i - 1) / 2 + j) * TPB] = pair_u<SH, T>(S, para, r2);
        }
    }
    pc[(SH::NE * (SH::NE - 1) / 2) * TPB] = T(0);
}

// Cache address of pair (e, j) for the moving electron e of sector SIG:
// pa = slot row of e (pairs with j < e at pa[j]), pb = column e (pairs with
// j > e at pb[j (j - 1) / 2]).  Partners of the other sector lie all below
// (SIG 1) or all above (SIG 0) e, so only same-sector partners select at
// run time; j == e lands on slot e (e + 1) / 2, a real pair or the zero slot.
template <class SH, int SIG, int TPB, int J, class T>
__device__ __forceinline__ T* pair_slot(T* pa, T* pb, int e) {
    constexpr bool other = (J < SH::NUP) != (SIG == 0);
    if (other) return SIG == 1 ? pa + J * TPB : pb + (J * (J - 1) / 2) * TPB;
    return J < e ? pa + J * TPB : pb + (J * (J - 1) / 2) * TPB;
}

// One-body (electron-nucleus) part of u at one position, summed over nuclei.
template <class SH, class T>
__device__ __forceinline__ T one_body_u(const SysT<SH, T>& S, T x, T y, T z) {
    T u = 0;
#pragma unroll
    for (int I = 0; I < SH::NNUC; ++I)
        u += pade_value(S.enA[I], S.enB[I], sq3(x - S.nuc[I][0], y - S.nuc[I][1], z - S.nuc[I][2]));
    return u;
}

// Change of u when electron e of sector SIG moves to (nx,ny,nz), with the
// old pair terms read from the cache and the old one-body term u1_old;
// un[j] receives the new pair terms, u1_new the new one-body term.
template <class SH, class T, int SIG, int TPB, class PosFn>
__device__ __forceinline__ T jastrow_delta_cached(const SysT<SH, T>& S, PosFn pos, T* pc, int e, T u1_old, T nx,
                                                  T ny, T nz, T (&un)[SH::NE], T& u1_new) {
    T* pa = pc + (e * (e - 1) / 2) * TPB;
    T* pb = pc + e * TPB;
    T du = 0;
    static_for<SH::NE>([&](auto jc) {
        constexpr int j = decltype(jc)::value;
        constexpr bool other = (j < SH::NUP) != (SIG == 0);
        const bool self = !other && j == e;
        const bool para = !other;
        T rb = sq3(nx - pos(j, 0), ny - pos(j, 1), nz - pos(j, 2));
        rb = self ? T(1) : rb;
        const T ub = pair_u<SH, T>(S, para, rb);
        un[j] = ub;
        const T ua = *pair_slot<SH, SIG, TPB, j>(pa, pb, e);
        du += self ? T(0) : ub - ua;
    });
    if (SH::JAS == JAS_PADE_EEN) {
        u1_new = one_body_u(S, nx, ny, nz);
        du -= u1_new - u1_old;
    }
    return du;
}

// Store the accepted move's pair terms un[j] (j != e) into the cache.
template <class SH, class T, int SIG, int TPB>
__device__ __forceinline__ void pair_cache_store(T* pc, int e, const T (&un)[SH::NE]) {
    T* pa = pc + (e * (e - 1) / 2) * TPB;
    T* pb = pc + e * TPB;
    static_for<SH::NE>([&](auto jc) {
        constexpr int j = decltype(jc)::value;
        constexpr bool other = (j < SH::NUP) != (SIG == 0);
        if (other || j != e) *pair_slot<SH, SIG, TPB, j>(pa, pb, e) = un[j];
    });
}

// ---------------------------------------------------------------------------
// Full evaluation of one configuration in precision TC.
// ---------------------------------------------------------------------------
template <class SH, class TC, int NR>
struct FullEval {
    double logabs;
    int sign;
    bool ok;
    TC el;
    TC gx[SH::NE], gy[SH::NE], gz[SH::NE], lap[SH::NE];   // grad psi/psi, lap psi/psi
    TC O[8 + (NR > 0 ? NR : 1)];
    TC dE[NR > 0 ? NR : 1];                               // d E_L / d theta_q (DEL evaluations)
};

// One spin sector.  With DEL (and NR > 0) it also accumulates into dErot the
// rotation-angle derivatives of the local energy: for column c of the sector
// rotated by theta_q, with B = A^-1, beta = B (d phi_c / d theta)(r_.),
//   d (X B)_ii = X_psi(r_i) B_ci - B_ci sum_k X_k(r_i) beta_k   (X = grad, lap),
//   d E_L / d theta_q += -1/2 sum_i [ d (L B)_ii + 2 d (G B)_ii . j_i ],
// j_i the Jastrow gradient of electron i (gjx, gjy, gjz).
template <class SH, class TC, int SIG, int NR, class DinvStore, bool DEL = false>
__device__ __forceinline__ void eval_sector(const SysT<SH, TC>& S, const TC (&r)[SH::NE][3], double& logdet,
                                            int& sg, bool& ok, TC (&gdx)[SH::NE], TC (&gdy)[SH::NE],
                                            TC (&gdz)[SH::NE], TC (&ld)[SH::NE], TC* Orot,
                                            DinvStore store, TC* omega, const TC* gjx = nullptr,
                                            const TC* gjy = nullptr, const TC* gjz = nullptr,
                                            TC* dErot = nullptr) {
    constexpr int NS = SIG == 0 ? SH::NUP : SH::NDN;
    if (NS == 0) return;
    constexpr int NSa = NS > 0 ? NS : 1;
    constexpr bool WD = DEL && NR > 0;
    constexpr int NRa = NR > 0 ? NR : 1;
    constexpr int NRD = WD ? NRa : 1;
    TC D[NSa][NSa], Gx[NSa][NSa], Gy[NSa][NSa], Gz[NSa][NSa], L[NSa][NSa];
    TC dvr[NSa][NRa];
    TC dgxr[NSa][NRD], dgyr[NSa][NRD], dgzr[NSa][NRD], dlr[NSa][NRD];
#pragma unroll 1
    for (int q = 0; q < NS; ++q) {
        const int e = SIG * SH::NUP + q;
        MOEval<SH, TC, SIG, WD ? 3 : 2, NR> m;
        m.run(S, r[e][0], r[e][1], r[e][2]);
#pragma unroll
        for (int k = 0; k < NS; ++k) { D[q][k] = m.v[k]; Gx[q][k] = m.gx[k]; Gy[q][k] = m.gy[k]; Gz[q][k] = m.gz[k]; L[q][k] = m.l[k]; }
#pragma unroll
        for (int qq = 0; qq < NR; ++qq) dvr[q][qq] = m.dv[qq];
        if constexpr (WD) {
#pragma unroll
            for (int qq = 0; qq < NR; ++qq) {
                dgxr[q][qq] = m.dgx[qq]; dgyr[q][qq] = m.dgy[qq]; dgzr[q][qq] = m.dgz[qq]; dlr[q][qq] = m.dl[qq];
            }
        }
    }
    TC Di[NSa][NSa];
    double lg;
    int s;
    ok = gj_inverse<NSa, TC>(D, Di, lg, s) && ok;
    logdet += lg;
    sg *= s;
#pragma unroll
    for (int k = 0; k < NS; ++k)
#pragma unroll
        for (int j = 0; j < NS; ++j) store(SIG, k, j, Di[k][j]);
#pragma unroll
    for (int q = 0; q < NS; ++q) {
        const int e = SIG * SH::NUP + q;
        TC ax = 0, ay = 0, az = 0, al = 0;
#pragma unroll
        for (int k = 0; k < NS; ++k) {
            TC w = Di[k][q];
            ax += Gx[q][k] * w; ay += Gy[q][k] * w; az += Gz[q][k] * w; al += L[q][k] * w;
        }
        gdx[e] = ax; gdy[e] = ay; gdz[e] = az; ld[e] = al;
    }
    if (NR > 0 && Orot) {
#pragma unroll
        for (int qq = 0; qq < NR; ++qq) {
            if (qq >= S.n_rot) continue;
            int c = S.rot_col[qq][SIG];
            TC acc = 0;
#pragma unroll
            for (int cc = 0; cc < NS; ++cc) {
                if (cc != c) continue;
#pragma unroll
                for (int row = 0; row < NS; ++row) acc += Di[cc][row] * dvr[row][qq];
            }
            Orot[qq] += acc;
        }
    }
    if constexpr (WD) {
#pragma unroll 1
        for (int qq = 0; qq < NR; ++qq) {
            if (qq >= S.n_rot) continue;
            const int c = S.rot_col[qq][SIG];
            if (c < 0) continue;
            TC beta[NSa];
#pragma unroll
            for (int col = 0; col < NS; ++col) {
                TC b = 0;
#pragma unroll
                for (int row = 0; row < NS; ++row) b += Di[col][row] * dvr[row][qq];
                beta[col] = b;
            }
            TC acc = 0;
#pragma unroll
            for (int q = 0; q < NS; ++q) {
                const int e = SIG * SH::NUP + q;
                TC bci = 0;
#pragma unroll
                for (int cc = 0; cc < NS; ++cc) bci = (cc == c) ? Di[cc][q] : bci;
                TC tx = 0, ty = 0, tz = 0, tl = 0;
#pragma unroll
                for (int col = 0; col < NS; ++col) {
                    tx += Gx[q][col] * beta[col]; ty += Gy[q][col] * beta[col];
                    tz += Gz[q][col] * beta[col]; tl += L[q][col] * beta[col];
                }
                const TC dgx = bci * (dgxr[q][qq] - tx), dgy = bci * (dgyr[q][qq] - ty);
                const TC dgz = bci * (dgzr[q][qq] - tz), dl = bci * (dlr[q][qq] - tl);
                acc += dl + 2 * (dgx * gjx[e] + dgy * gjy[e] + dgz * gjz[e]);
            }
            dErot[qq] += TC(-0.5) * acc;
        }
    }
    if (omega) {
        // d ln|D| / dR_I = -sum_rows sum_k Dinv[k][row] sum_{a on I} C[k][a] grad chi_a(r_row)
#pragma unroll 1
        for (int q = 0; q < NS; ++q) {
            const int e = SIG * SH::NUP + q;
#pragma unroll
            for (int I = 0; I < SH::NNUC; ++I) {
                MOEval<SH, TC, SIG, 1, 0> m;
                m.run(S, r[e][0], r[e][1], r[e][2], I);
                TC ox = 0, oy = 0, oz = 0;
#pragma unroll
                for (int k = 0; k < NS; ++k) { ox += Di[k][q] * m.gx[k]; oy += Di[k][q] * m.gy[k]; oz += Di[k][q] * m.gz[k]; }
                omega[3 * I] -= ox; omega[3 * I + 1] -= oy; omega[3 * I + 2] -= oz;
            }
        }
    }
}

// Jastrow over all pairs: u, grad_i u (true gradient), sum_j (u''+2u'/r),
// sum_j u'^2 (for the per-pair Laplacian quirk), parameter derivatives, and
// the Coulomb potential V_ee + V_en + V_nn from the same distances (one
// reciprocal square root per pair).
template <class SH, class TC, bool WANT_O>
__device__ __forceinline__ TC jastrow_coulomb(const SysT<SH, TC>& S, const TC (&r)[SH::NE][3], TC (&gx)[SH::NE],
                                              TC (&gy)[SH::NE], TC (&gz)[SH::NE], TC (&lu)[SH::NE],
                                              TC (&gsq)[SH::NE], TC* O, TC& V) {
    TC u = 0;
    V = S.v_nn;
#pragma unroll
    for (int i = 0; i < SH::NE; ++i) { gx[i] = 0; gy[i] = 0; gz[i] = 0; lu[i] = 0; gsq[i] = 0; }
#pragma unroll
    for (int i = 0; i < SH::NE; ++i)
#pragma unroll
        for (int j = i + 1; j < SH::NE; ++j) {
            const bool para = ((i < SH::NUP) == (j < SH::NUP));
            TC dx = r[i][0] - r[j][0], dy = r[i][1] - r[j][1], dz = r[i][2] - r[j][2];
            TC d, ri;
            dist(dx * dx + dy * dy + dz * dz, d, ri);
            V += ri;
            if (SH::JAS == JAS_NONE) continue;
            TC uu, upr, lt;
            const int c = para ? 1 : 0;
            if (SH::JAS == JAS_PADE_F) pade_f(S.F, S.invF, d, ri, uu, upr, lt);
            else pade_ab(S.a_ee[c], S.b_ee[c], d, ri, uu, upr, lt);
            u += uu;
            bool skip = (SH::JAS == JAS_PADE_EEN) ? (d < TC(1e-10)) : (d == TC(0));
            if (!skip) {
                gx[i] += upr * dx; gy[i] += upr * dy; gz[i] += upr * dz;
                gx[j] -= upr * dx; gy[j] -= upr * dy; gz[j] -= upr * dz;
                lu[i] += lt; lu[j] += lt;
                TC up = upr * d;
                gsq[i] += up * up; gsq[j] += up * up;
            }
            if (WANT_O && SH::JAS == JAS_PADE_EEN) {
                TC inv = TC(1) / (1 + S.b_ee[c] * d);
                O[c] += -S.a_ee[c] * d * d * inv * inv;
                O[2 + c] += d * inv;
            }
        }
#pragma unroll
    for (int i = 0; i < SH::NE; ++i)
#pragma unroll
        for (int I = 0; I < SH::NNUC; ++I) {
            TC dx = r[i][0] - S.nuc[I][0], dy = r[i][1] - S.nuc[I][1], dz = r[i][2] - S.nuc[I][2];
            TC d, ri;
            dist(dx * dx + dy * dy + dz * dz, d, ri);
            V -= S.Z[I] * ri;
            if (SH::JAS != JAS_PADE_EEN) continue;
            TC uu, upr, lt;
            pade_ab(S.enA[I], S.enB[I], d, ri, uu, upr, lt);
            u -= uu;
            if (!(d < TC(1e-10))) {
                gx[i] -= upr * dx; gy[i] -= upr * dy; gz[i] -= upr * dz;
                lu[i] -= lt;
            }
            if (WANT_O) {
                TC inv = TC(1) / (1 + S.enB[I] * d);
                TC dB = S.Aspec[I] * S.Z[I] * d * d * inv * inv;
                TC dA = -S.Z[I] * d * inv;
                if (S.species[I] == 0) { O[4] += dB; O[6] += dA; }
                else { O[5] += dB; O[7] += dA; }
            }
        }
    return u;
}

template <class SH, class TC, int NR, class DinvStore, bool DEL = false>
__device__ __forceinline__ void evaluate_config(const SysT<SH, TC>& S, const TC (&r)[SH::NE][3],
                                                FullEval<SH, TC, NR>& out, bool want_o, DinvStore store,
                                                TC* omega) {
    TC gjx[SH::NE], gjy[SH::NE], gjz[SH::NE], lu[SH::NE], gsq[SH::NE];
#pragma unroll
    for (int p = 0; p < 8 + (NR > 0 ? NR : 1); ++p) out.O[p] = 0;
    TC u, V;
    if (NR > 0 || want_o) u = jastrow_coulomb<SH, TC, true>(S, r, gjx, gjy, gjz, lu, gsq, out.O, V);
    else u = jastrow_coulomb<SH, TC, false>(S, r, gjx, gjy, gjz, lu, gsq, out.O, V);
    TC gdx[SH::NE], gdy[SH::NE], gdz[SH::NE], ld[SH::NE];
    double logdet = 0.0;
    int sg = 1;
    bool ok = true;
#pragma unroll
    for (int q = 0; q < (NR > 0 ? NR : 1); ++q) out.dE[q] = 0;
    eval_sector<SH, TC, 0, NR, DinvStore, DEL>(S, r, logdet, sg, ok, gdx, gdy, gdz, ld, out.O + 8, store, omega, gjx,
                                              gjy, gjz, out.dE);
    eval_sector<SH, TC, 1, NR, DinvStore, DEL>(S, r, logdet, sg, ok, gdx, gdy, gdz, ld, out.O + 8, store, omega, gjx,
                                              gjy, gjz, out.dE);
    TC kin = 0;
#pragma unroll
    for (int e = 0; e < SH::NE; ++e) {
        TC ax = S.qa * gjx[e], ay = S.qa * gjy[e], az = S.qa * gjz[e];
        TC lj = S.quirk_lap ? (lu[e] + gsq[e]) : (lu[e] + gjx[e] * gjx[e] + gjy[e] * gjy[e] + gjz[e] * gjz[e]);
        TC lp = ld[e] + 2 * (gdx[e] * ax + gdy[e] * ay + gdz[e] * az) + lj;
        out.gx[e] = gdx[e] + ax; out.gy[e] = gdy[e] + ay; out.gz[e] = gdz[e] + az;
        out.lap[e] = lp;
        kin += lp;
    }
    out.el = TC(-0.5) * kin + V;
    out.logabs = logdet + (double)u;
    out.sign = sg;
    out.ok = ok;
}

// ---------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------
template <class SH, class TS>
__global__ void k_init(const __grid_constant__ SysT<SH, double> S, TS* __restrict__ pos, int W, int Wcap,
                       uint64_t seed) {
    int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= W) return;
#pragma unroll
    for (int e = 0; e < SH::NE; ++e) {
        U4 x = rng_draw(seed, (uint32_t)w, 0, (uint32_t)S.perm[e], TAG_INIT);
        double n0, n1, n2, n3;
        bm(x.x, x.y, n0, n1);
        bm(x.z, x.w, n2, n3);
        int c = S.init_nuc[e];
        double cx = c >= 0 ? S.nuc[c][0] : 0.0, cy = c >= 0 ? S.nuc[c][1] : 0.0, cz = c >= 0 ? S.nuc[c][2] : 0.0;
        pos[(3 * e + 0) * (size_t)Wcap + w] = (TS)(cx + S.init_sigma * n0);
        pos[(3 * e + 1) * (size_t)Wcap + w] = (TS)(cy + S.init_sigma * n1);
        pos[(3 * e + 2) * (size_t)Wcap + w] = (TS)(cz + S.init_sigma * n2);
    }
}

// Full evaluation of walker w (refresh of the inverse, log|psi|, E_L and the
// requested extras); returns E_L (0 for an inactive lane, which still runs the
// arithmetic on a dummy configuration so that the block stays converged).
template <class SH, class TC, class TS, int NR, bool DEL = false>
__device__ __forceinline__ double measure_walker(const SysT<SH, TC>& S, const TS* __restrict__ pos,
                                                 TS* __restrict__ dinv, double* __restrict__ logabs,
                                                 int* __restrict__ sign, double* __restrict__ el, int w, bool act,
                                                 int Wcap, int write_state, const MeasureOut& out, int P,
                                                 int* flags) {
    TC r[SH::NE][3];
#pragma unroll
    for (int e = 0; e < SH::NE; ++e)
#pragma unroll
        for (int c = 0; c < 3; ++c) r[e][c] = act ? (TC)pos[(3 * e + c) * (size_t)Wcap + w] : TC(e + 1) * TC(0.37 + c);
    constexpr int NM = SH::NMAX;
    auto store = [&](int sig, int k, int j, TC v) {
        if (act && write_state) dinv[((size_t)(sig * NM * NM + k * NM + j)) * Wcap + w] = (TS)v;
    };
    TC omega[3 * SH::NNUC];
#pragma unroll
    for (int i = 0; i < 3 * SH::NNUC; ++i) omega[i] = 0;
    FullEval<SH, TC, NR> ev;
    evaluate_config<SH, TC, NR, decltype(store), DEL>(S, r, ev, out.O != nullptr, store,
                                                      (act && out.omega) ? omega : (TC*)nullptr);
    double e_l = (double)ev.el;
    if (act) {
        int fl = 0;
        if (!ev.ok) fl |= FLAG_SINGULAR;
        if (!isfinite(e_l)) fl |= FLAG_NONFINITE;
        if (fl) atomicOr(flags, fl);
        if (write_state) { logabs[w] = ev.logabs; sign[w] = ev.sign; el[w] = e_l; }
        if (out.grad) {
#pragma unroll
            for (int e = 0; e < SH::NE; ++e) {
                out.grad[((size_t)w * SH::NE + e) * 3 + 0] = (double)ev.gx[e];
                out.grad[((size_t)w * SH::NE + e) * 3 + 1] = (double)ev.gy[e];
                out.grad[((size_t)w * SH::NE + e) * 3 + 2] = (double)ev.gz[e];
            }
        }
        if (out.lap) {
#pragma unroll
            for (int e = 0; e < SH::NE; ++e) out.lap[(size_t)w * SH::NE + e] = (double)ev.lap[e];
        }
        if (out.O) {
            for (int p = 0; p < P; ++p) out.O[(size_t)w * P + p] = (double)ev.O[p];
        }
        if (DEL && out.dEL) {
            // rotation columns; the Jastrow columns 0..7 come from k_jastrow3_logderiv
            for (int p = 8; p < P; ++p) out.dEL[(size_t)w * P + p] = (double)ev.dE[p - 8];
        }
        if (out.fhf) {
#pragma unroll
            for (int I = 0; I < SH::NNUC; ++I) {
                TC fx = 0, fy = 0, fz = 0;
#pragma unroll
                for (int i = 0; i < SH::NE; ++i) {
                    TC dx = r[i][0] - S.nuc[I][0], dy = r[i][1] - S.nuc[I][1], dz = r[i][2] - S.nuc[I][2];
                    TC d = fsqrt(dx * dx + dy * dy + dz * dz);
                    if (d > TC(1e-10)) { TC f = S.Z[I] / (d * d * d); fx += f * dx; fy += f * dy; fz += f * dz; }
                }
#pragma unroll
                for (int J = 0; J < SH::NNUC; ++J) {
                    if (J == I) continue;
                    TC dx = S.nuc[I][0] - S.nuc[J][0], dy = S.nuc[I][1] - S.nuc[J][1], dz = S.nuc[I][2] - S.nuc[J][2];
                    TC d = fsqrt(dx * dx + dy * dy + dz * dz);
                    if (d > TC(1e-10)) { TC f = S.Z[I] * S.Z[J] / (d * d * d); fx -= f * dx; fy -= f * dy; fz -= f * dz; }
                }
                out.fhf[((size_t)w * SH::NNUC + I) * 3 + 0] = (double)fx;
                out.fhf[((size_t)w * SH::NNUC + I) * 3 + 1] = (double)fy;
                out.fhf[((size_t)w * SH::NNUC + I) * 3 + 2] = (double)fz;
            }
        }
        if (out.omega) {
            if (SH::JAS == JAS_PADE_EEN) {
#pragma unroll
                for (int I = 0; I < SH::NNUC; ++I)
#pragma unroll
                    for (int i = 0; i < SH::NE; ++i) {
                        TC dx = r[i][0] - S.nuc[I][0], dy = r[i][1] - S.nuc[I][1], dz = r[i][2] - S.nuc[I][2];
                        TC d = fsqrt(dx * dx + dy * dy + dz * dz);
                        if (d < TC(1e-10)) continue;
                        TC den = 1 + S.enB[I] * d;
                        TC f = S.enA[I] / (d * den * den);
                        omega[3 * I] += f * dx; omega[3 * I + 1] += f * dy; omega[3 * I + 2] += f * dz;
                    }
            }
#pragma unroll
            for (int i = 0; i < 3 * SH::NNUC; ++i) out.omega[(size_t)w * 3 * SH::NNUC + i] = (double)omega[i];
        }
    }
    return act ? e_l : 0.0;
}

template <class SH, class TC, class TS, int TPB, int NR, bool DEL = false>
__global__ void __launch_bounds__(TPB) k_measure(const __grid_constant__ SysT<SH, TC> S,
                                                 const TS* __restrict__ pos, TS* __restrict__ dinv,
                                                 double* __restrict__ logabs, int* __restrict__ sign,
                                                 double* __restrict__ el, int W, int Wcap, int write_state,
                                                 MeasureOut out, int P, double* partial, int* flags) {
    const int w = blockIdx.x * TPB + threadIdx.x;
    double e_l = measure_walker<SH, TC, TS, NR, DEL>(S, pos, dinv, logabs, sign, el, w, w < W, Wcap, write_state,
                                                     out, P, flags);
    if (partial) block_partial<TPB>(e_l, partial, blockIdx.x);
}

// Bytes of a system table staged in shared memory (16-byte multiple).
template <class SH, class T>
__host__ __device__ constexpr size_t batch_table_bytes() {
    return (sizeof(SysT<SH, T>) + 15) / 16 * 16;
}

// ---------------------------------------------------------------------------
// Two-pass refresh of FP32 walkers in float-float arithmetic.
// Pass 1, one thread per (walker, electron): the electron's MO row (values,
// gradients, Laplacians) and its Jastrow and Coulomb sums (pairs seen from
// both ends, halved), stored as float-float pairs in rows[e][quantity][Wcap].
// Pass 2, one thread per walker: Gauss-Jordan inverse of each sector's
// Slater matrix from the stored rows, the inverse written back for the
// sweeps, the kinetic contractions and E_L.  Each pass is a short
// instruction stream, so the FP32 pipe is not starved by instruction fetch
// as a single fully unrolled per-walker kernel is.
// ---------------------------------------------------------------------------
template <class SH>
struct RowLayout {
    static constexpr int NM = SH::NMAX;
    // v, d/dx, d/dy, d/dz, lap (NM each), then Jastrow gx, gy, gz, lap u,
    // |grad u_pair|^2 sum, u (halved pairs), V (halved pairs)
    static constexpr int QN = 5 * NM + 7;
    static constexpr int J0 = 5 * NM;
};

// Values, gradients and Laplacians of the NM orbitals of sector sig at one
// position, for Gaussian bases, with rolled loops over nuclei, shells,
// primitives and AOs: a single copy of the AO -> MO contraction, so that the
// instruction stream of the float-float refresh stays cache-resident.  The
// AO formulas are MOEval's (src/systems/methane.rs:498-590).
template <class SH, int MODE>
__device__ __forceinline__ void orbitals_gto_rolled(const SysT<SH, ff>& S, int sig, ff x, ff y, ff z,
                                                    ff (&v)[SH::NMAX], ff (&gx)[SH::NMAX], ff (&gy)[SH::NMAX],
                                                    ff (&gz)[SH::NMAX], ff (&l)[SH::NMAX]) {
    constexpr int NM = SH::NMAX;
#pragma unroll
    for (int k = 0; k < NM; ++k) { v[k] = 0; gx[k] = 0; gy[k] = 0; gz[k] = 0; l[k] = 0; }
#pragma unroll 1
    for (int I = 0; I < SH::NNUC; ++I) {
        const ff dx = x - S.nuc[I][0], dy = y - S.nuc[I][1], dz = z - S.nuc[I][2];
        const ff r2 = dx * dx + dy * dy + dz * dz;
#pragma unroll 1
        for (int sh = S.sh_start[I]; sh < S.sh_start[I + 1]; ++sh) {
            const int p0 = S.sh_p0[sh], p1 = p0 + S.sh_np[sh];
            const int s0 = S.sh_s0[sh], s1 = S.sh_s1[sh], pa = S.sh_p[sh];
            // radial sums R0 = sum c e, R1 = sum c al e, R2 = sum c al^2 e of
            // the shell's s0, s1 and p coefficient sets (warp-uniform skips
            // of the sets a shell does not have)
            ff a0 = 0, a1 = 0, ap = 0, b0 = 0, b1 = 0, bp = 0, c0 = 0, c1 = 0, cpp = 0;
#pragma unroll 1
            for (int p = p0; p < p1; ++p) {
                const ff al = S.pexp[p];
                const ff e = fexp(-al * r2);
                if (s0 >= 0) ff_fma_lazy(a0, S.cs0[p], e);
                if (s1 >= 0) ff_fma_lazy(a1, S.cs1[p], e);
                if (pa >= 0) ff_fma_lazy(ap, S.cp[p], e);
                if (MODE >= 2) {
                    const ff ea = al * e, eaa = al * ea;
                    if (s0 >= 0) { ff_fma_lazy(b0, S.cs0[p], ea); ff_fma_lazy(c0, S.cs0[p], eaa); }
                    if (s1 >= 0) { ff_fma_lazy(b1, S.cs1[p], ea); ff_fma_lazy(c1, S.cs1[p], eaa); }
                    if (pa >= 0) { ff_fma_lazy(bp, S.cp[p], ea); ff_fma_lazy(cpp, S.cp[p], eaa); }
                }
            }
            a0 = ff_norm(a0); b0 = ff_norm(b0); c0 = ff_norm(c0);
            a1 = ff_norm(a1); b1 = ff_norm(b1); c1 = ff_norm(c1);
            ap = ff_norm(ap); bp = ff_norm(bp); cpp = ff_norm(cpp);
            const ff lp = ff(-10.0f) * bp + ff(4.0f) * r2 * cpp;
#pragma unroll 1
            for (int m = 0; m < 5; ++m) {
                const int a = m == 0 ? s0 : (m == 1 ? s1 : (pa >= 0 ? pa + m - 2 : -1));
                if (a < 0) continue;
                ff chi, ax, ay, az, la;
                if (m < 2) {
                    // s AO: chi = R0, grad = -2 R1 dr, lap = -6 R1 + 4 r^2 R2
                    const ff A = m == 0 ? a0 : a1, B = m == 0 ? b0 : b1, C = m == 0 ? c0 : c1;
                    const ff t = ff(-2.0f) * B;
                    chi = A; ax = t * dx; ay = t * dy; az = t * dz;
                    la = ff(-6.0f) * B + ff(4.0f) * r2 * C;
                } else {
                    // p AO along axis m - 2: chi = x_m R(r), grad = x_m (-2 R1 dr) + e_m R0,
                    // lap = x_m (-10 R1 + 4 r^2 R2)
                    const ff xm = m == 2 ? dx : (m == 3 ? dy : dz);
                    const ff t = ff(-2.0f) * bp * xm;
                    chi = xm * ap;
                    ax = t * dx + (m == 2 ? ap : ff(0.0f));
                    ay = t * dy + (m == 3 ? ap : ff(0.0f));
                    az = t * dz + (m == 4 ? ap : ff(0.0f));
                    la = xm * lp;
                }
#pragma unroll
                for (int k = 0; k < NM; ++k) {
                    const ff c = S.C[sig][a][k];
                    ff_fma_lazy(v[k], c, chi);
                    if (MODE >= 2) {
                        ff_fma_lazy(gx[k], c, ax);
                        ff_fma_lazy(gy[k], c, ay);
                        ff_fma_lazy(gz[k], c, az);
                        ff_fma_lazy(l[k], c, la);
                    }
                }
            }
        }
    }
#pragma unroll
    for (int k = 0; k < NM; ++k) {
        v[k] = ff_norm(v[k]); gx[k] = ff_norm(gx[k]); gy[k] = ff_norm(gy[k]); gz[k] = ff_norm(gz[k]);
        l[k] = ff_norm(l[k]);
    }
}

template <class SH, int SIG, int MODE>
__device__ __forceinline__ void rows_orbitals(const SysT<SH, ff>& S, ff x, ff y, ff z, ff (&v)[SH::NMAX],
                                              ff (&gx)[SH::NMAX], ff (&gy)[SH::NMAX], ff (&gz)[SH::NMAX],
                                              ff (&l)[SH::NMAX]) {
    MOEval<SH, ff, SIG, MODE, 0> m;
    m.run(S, x, y, z);
#pragma unroll
    for (int k = 0; k < SH::NMAX; ++k) { v[k] = m.v[k]; gx[k] = m.gx[k]; gy[k] = m.gy[k]; gz[k] = m.gz[k]; l[k] = m.l[k]; }
}

// Pass 1 for electron e (sector sig) of walker w.  VALUES: only the orbital
// values and the Jastrow u (what the inverse and log|psi| need).
template <class SH, class TS, bool VALUES>
__device__ __forceinline__ void rows_electron(const SysT<SH, ff>& S, const TS* __restrict__ pos,
                                             float2* __restrict__ rows, int e, int w, int Wcap) {
    constexpr int MODE = VALUES ? 0 : 2;
    using RL = RowLayout<SH>;
    constexpr int NM = RL::NM;
    const size_t st = (size_t)Wcap;
    const int sig = e < SH::NUP ? 0 : 1;
    float2* out = rows + (size_t)e * RL::QN * st + w;
    const ff x = ff((float)pos[(3 * e + 0) * st + w]), y = ff((float)pos[(3 * e + 1) * st + w]),
             z = ff((float)pos[(3 * e + 2) * st + w]);
    {
        ff v[NM], ogx[NM], ogy[NM], ogz[NM], ol[NM];
        if constexpr (SH::BASIS == BASIS_GTO) {
            orbitals_gto_rolled<SH, MODE>(S, sig, x, y, z, v, ogx, ogy, ogz, ol);
        } else {
            if (sig == 0) rows_orbitals<SH, 0, MODE>(S, x, y, z, v, ogx, ogy, ogz, ol);
            else rows_orbitals<SH, 1, MODE>(S, x, y, z, v, ogx, ogy, ogz, ol);
        }
#pragma unroll
        for (int k = 0; k < NM; ++k) {
            ff_store(out + (0 * NM + k) * st, v[k]);
            if (VALUES) continue;
            ff_store(out + (1 * NM + k) * st, ogx[k]);
            ff_store(out + (2 * NM + k) * st, ogy[k]);
            ff_store(out + (3 * NM + k) * st, ogz[k]);
            ff_store(out + (4 * NM + k) * st, ol[k]);
        }
    }
    ff gx = 0, gy = 0, gz = 0, lu = 0, gsq = 0, u = 0, V = 0;
#pragma unroll 1
    for (int j = 0; j < SH::NE; ++j) {
        if (j == e) continue;
        const ff dx = x - ff((float)pos[(3 * j + 0) * st + w]), dy = y - ff((float)pos[(3 * j + 1) * st + w]),
                 dz = z - ff((float)pos[(3 * j + 2) * st + w]);
        ff d, ri;
        dist(dx * dx + dy * dy + dz * dz, d, ri);
        V += ff(0.5f) * ri;
        if (SH::JAS == JAS_NONE) continue;
        ff uu, upr, lt;
        if (SH::JAS == JAS_PADE_F) {
            pade_f(S.F, S.invF, d, ri, uu, upr, lt);
        } else {
            const int c = ((j < SH::NUP) == (e < SH::NUP)) ? 1 : 0;
            pade_ab(S.a_ee[c], S.b_ee[c], d, ri, uu, upr, lt);
        }
        u += ff(0.5f) * uu;
        const bool skip = (SH::JAS == JAS_PADE_EEN) ? (d < ff(1e-10)) : (d == ff(0));
        if (!VALUES && !skip) {
            gx += upr * dx; gy += upr * dy; gz += upr * dz;
            lu += lt;
            const ff up = upr * d;
            gsq += up * up;
        }
    }
#pragma unroll 1
    for (int I = 0; I < SH::NNUC; ++I) {
        const ff dx = x - S.nuc[I][0], dy = y - S.nuc[I][1], dz = z - S.nuc[I][2];
        ff d, ri;
        dist(dx * dx + dy * dy + dz * dz, d, ri);
        V -= S.Z[I] * ri;
        if (SH::JAS != JAS_PADE_EEN) continue;
        ff uu, upr, lt;
        pade_ab(S.enA[I], S.enB[I], d, ri, uu, upr, lt);
        u -= uu;
        if (!VALUES && !(d < ff(1e-10))) {
            gx -= upr * dx; gy -= upr * dy; gz -= upr * dz;
            lu -= lt;
        }
    }
    if (VALUES) {
        ff_store(out + (RL::J0 + 5) * st, u);
        return;
    }
    ff_store(out + (RL::J0 + 0) * st, gx);
    ff_store(out + (RL::J0 + 1) * st, gy);
    ff_store(out + (RL::J0 + 2) * st, gz);
    ff_store(out + (RL::J0 + 3) * st, lu);
    ff_store(out + (RL::J0 + 4) * st, gsq);
    ff_store(out + (RL::J0 + 5) * st, u);
    ff_store(out + (RL::J0 + 6) * st, V);
}

// One spin sector (NS electrons, runtime sector index sig) of pass 2.
template <class SH, class TS, int NS, bool VALUES>
__device__ __forceinline__ void assemble_sector(const SysT<SH, ff>& S, const float2* __restrict__ rows,
                                                TS* __restrict__ dinv, int SIG, int w, int wr, bool act, int Wcap,
                                                int write_state, ff& pm, int& pe, int& sg, bool& ok, ff& kin,
                                                ff& ut, ff& vt) {
    using RL = RowLayout<SH>;
    constexpr int NM = RL::NM;
    if (NS == 0) return;
    constexpr int NSa = NS > 0 ? NS : 1;
    const size_t st = (size_t)Wcap;
    ff D[NSa][NSa], Di[NSa][NSa];
#pragma unroll
    for (int q = 0; q < NS; ++q)
#pragma unroll
        for (int k = 0; k < NS; ++k) D[q][k] = ff_load(rows + ((size_t)(SIG * SH::NUP + q) * RL::QN + k) * st + wr);
    int s = 1;
    ok = gj_inverse_prod<NSa>(D, Di, pm, pe, s) && ok;
    sg *= s;
    if (act && write_state) {
#pragma unroll
        for (int k = 0; k < NS; ++k)
#pragma unroll
            for (int j = 0; j < NS; ++j) dinv[((size_t)(SIG * NM * NM + k * NM + j)) * Wcap + w] = (TS)Di[k][j];
    }
    if constexpr (VALUES) {
#pragma unroll
        for (int q = 0; q < NS; ++q) ut += ff_load(rows + ((size_t)(SIG * SH::NUP + q) * RL::QN + RL::J0 + 5) * st + wr);
        return;
    }
#pragma unroll
    for (int q = 0; q < NS; ++q) {
        const float2* r = rows + (size_t)(SIG * SH::NUP + q) * RL::QN * st + wr;
        ff gdx = 0, gdy = 0, gdz = 0, ld = 0;
#pragma unroll
        for (int k = 0; k < NS; ++k) {
            const ff dk = Di[k][q];
            gdx += ff_load(r + (1 * NM + k) * st) * dk;
            gdy += ff_load(r + (2 * NM + k) * st) * dk;
            gdz += ff_load(r + (3 * NM + k) * st) * dk;
            ld += ff_load(r + (4 * NM + k) * st) * dk;
        }
        const ff gjx = ff_load(r + (RL::J0 + 0) * st), gjy = ff_load(r + (RL::J0 + 1) * st),
                 gjz = ff_load(r + (RL::J0 + 2) * st), lu = ff_load(r + (RL::J0 + 3) * st),
                 gsq = ff_load(r + (RL::J0 + 4) * st);
        const ff ax = S.qa * gjx, ay = S.qa * gjy, az = S.qa * gjz;
        const ff lj = S.quirk_lap ? (lu + gsq) : (lu + gjx * gjx + gjy * gjy + gjz * gjz);
        kin += ld + 2 * (gdx * ax + gdy * ay + gdz * az) + lj;
        ut += ff_load(r + (RL::J0 + 5) * st);
        vt += ff_load(r + (RL::J0 + 6) * st);
    }
}

// Pass 2 for walker w (inactive lanes read walker 0's rows and store nothing).
template <class SH, class TS, bool VALUES>
__device__ __forceinline__ double assemble_walker(const SysT<SH, ff>& S, const float2* __restrict__ rows,
                                                  TS* __restrict__ dinv, double* __restrict__ logabs,
                                                  int* __restrict__ sign, double* __restrict__ el, int w, bool act,
                                                  int Wcap, int write_state, int* flags) {
    const int wr = act ? w : 0;
    ff pm = ff(1.0f), kin = 0, ut = 0, vt = 0;
    int pe = 0, sg = 1;
    bool ok = true;
    if constexpr (SH::NUP == SH::NDN) {
        // equal sectors share one copy of the sector code (a short
        // instruction stream keeps the FP32 pipe fed from the cache)
#pragma unroll 1
        for (int sig = 0; sig < 2; ++sig)
            assemble_sector<SH, TS, SH::NUP, VALUES>(S, rows, dinv, sig, w, wr, act, Wcap, write_state, pm, pe, sg,
                                                     ok, kin, ut, vt);
    } else {
        assemble_sector<SH, TS, SH::NUP, VALUES>(S, rows, dinv, 0, w, wr, act, Wcap, write_state, pm, pe, sg, ok, kin,
                                                 ut, vt);
        assemble_sector<SH, TS, SH::NDN, VALUES>(S, rows, dinv, 1, w, wr, act, Wcap, write_state, pm, pe, sg, ok, kin,
                                                 ut, vt);
    }
    const double logdet = log((double)pm) + (double)pe * 0.6931471805599453;
    const double e_l = VALUES ? 0.0 : (double)(ff(-0.5f) * kin + vt + S.v_nn);
    if (!act) return 0.0;
    int fl = 0;
    if (!ok) fl |= FLAG_SINGULAR;
    if (!isfinite(e_l) || !isfinite(logdet)) fl |= FLAG_NONFINITE;
    if (fl) atomicOr(flags, fl);
    if (write_state) {
        logabs[w] = logdet + (double)ut;
        sign[w] = sg;
        if (!VALUES) el[w] = e_l;
    }
    return e_l;
}

template <class SH, class TS, bool VALUES>
__global__ void __launch_bounds__(128) k_rows(const __grid_constant__ SysT<SH, ff> S, const TS* __restrict__ pos,
                                              float2* __restrict__ rows, int W, int Wcap) {
    const int w = blockIdx.x * 128 + threadIdx.x;
    const int e = blockIdx.y;
    if (w >= W) return;
    rows_electron<SH, TS, VALUES>(S, pos, rows, e, w, Wcap);
}

template <class SH, class TS, int TPB, bool VALUES>
__global__ void __launch_bounds__(TPB) k_assemble(const __grid_constant__ SysT<SH, ff> S,
                                                  const float2* __restrict__ rows, TS* __restrict__ dinv,
                                                  double* __restrict__ logabs, int* __restrict__ sign,
                                                  double* __restrict__ el, int W, int Wcap, int write_state,
                                                  double* partial, int* flags) {
    const int w = blockIdx.x * TPB + threadIdx.x;
    const double e_l = assemble_walker<SH, TS, VALUES>(S, rows, dinv, logabs, sign, el, w, w < W, Wcap, write_state,
                                                       flags);
    if (!VALUES && partial) block_partial<TPB>(e_l, partial, blockIdx.x);
}

// Batched forms.  Pass 1 runs over (tile, electron) items in tile-major
// order so consecutive items of a block share their system's table.
template <class SH, class TS, int TPB>
__global__ void __launch_bounds__(TPB) kb_rows(const BatchTile* __restrict__ tiles, int ntiles,
                                               const BatchRec* __restrict__ recs) {
    __shared__ __align__(16) unsigned char sraw[batch_table_bytes<SH, ff>()];
    SysT<SH, ff>& S = *reinterpret_cast<SysT<SH, ff>*>(sraw);
    int t0, t1;
    batch_tile_range(ntiles * SH::NE, t0, t1);
    int cur = -1;
    for (int it = t0; it < t1; ++it) {
        const int ti = it / SH::NE, e = it - ti * SH::NE;
        const BatchTile tl = tiles[ti];
        if (tl.rec != cur) {
            __syncthreads();
            stage_table(&S, recs[tl.rec].tab_d);
            __syncthreads();
            cur = tl.rec;
        }
        const BatchRec& R = recs[tl.rec];
        const int w = tl.w0 + (int)threadIdx.x;
        if (w < R.W) rows_electron<SH, TS, false>(S, (const TS*)R.pos, R.rows, e, w, R.Wcap);
    }
}

template <class SH, class TS, int TPB>
__global__ void __launch_bounds__(TPB) kb_assemble(const BatchTile* __restrict__ tiles, int ntiles,
                                                   const BatchRec* __restrict__ recs, double* tile_partial) {
    __shared__ __align__(16) unsigned char sraw[batch_table_bytes<SH, ff>()];
    SysT<SH, ff>& S = *reinterpret_cast<SysT<SH, ff>*>(sraw);
    int t0, t1;
    batch_tile_range(ntiles, t0, t1);
    int cur = -1;
    for (int ti = t0; ti < t1; ++ti) {
        const BatchTile tl = tiles[ti];
        if (tl.rec != cur) {
            stage_table(&S, recs[tl.rec].tab_d);   // block_partial ended the previous tile with a barrier
            __syncthreads();
            cur = tl.rec;
        }
        const BatchRec& R = recs[tl.rec];
        const int w = tl.w0 + (int)threadIdx.x;
        const double e_l = assemble_walker<SH, TS, false>(S, R.rows, (TS*)R.dinv, R.logabs, R.sign, R.el, w,
                                                          w < R.W, R.Wcap, 1, R.flags);
        block_partial<TPB>(e_l, tile_partial, ti);
    }
}

template <class T> struct Vec2T;
template <> struct Vec2T<float> { using type = float2; };
template <> struct Vec2T<double> { using type = double2; };

// Walker positions in shared memory: (x, y) pairs [NE][TPB] (one 64-bit
// access per electron, 128-bit for FP64) followed by z [NE][TPB].
template <class T, int TPB, int NE>
struct PosCols {
    using V2 = typename Vec2T<T>::type;
    V2* xy;
    T* zz;
    int t;
    __device__ __forceinline__ PosCols(T* base, int t_)
        : xy(reinterpret_cast<V2*>(base)), zz(base + 2 * NE * TPB), t(t_) {}
    __device__ __forceinline__ T operator()(int j, int c) const {
        if (c == 2) return zz[j * TPB + t];
        const V2 v = xy[j * TPB + t];
        return c == 0 ? v.x : v.y;
    }
    __device__ __forceinline__ void set(int j, T x, T y, T z) const {
        V2 v;
        v.x = x;
        v.y = y;
        xy[j * TPB + t] = v;
        zz[j * TPB + t] = z;
    }
};

// Single-electron sweeps.  Shared memory holds the block's walkers as
// structure-of-arrays columns: positions (PosCols, 3 NE words), inverse Slater
// matrices [2][NMAX^2][TPB]; each thread only touches its own column, so no
// barrier is needed.
template <class SH, class T, int SIG, int MOVE, int TPB>
__device__ __forceinline__ void sweep_sector(const SysT<SH, T>& S, T* sp, T* sd, T* pc, T* u1c, int t, uint32_t w,
                                             uint64_t st, uint64_t seed, T step, T tau, T maxd, int fixed_node,
                                             int& sgn, unsigned& acc, int& flg) {
    constexpr int NS = SIG == 0 ? SH::NUP : SH::NDN;
    constexpr int NM = SH::NMAX;
    constexpr bool PAIRS = sweep_pairs<SH, MOVE>() > 0;
    const PosCols<T, TPB, SH::NE> P(sp, t);
#define DI(k, j) sd[((SIG * NM * NM) + (k) * NM + (j)) * TPB + t]
    for (int q = 0; q < NS; ++q) {
        const int e = SIG * SH::NUP + q;
        T rx = P(e, 0), ry = P(e, 1), rz = P(e, 2);
        T mv[NM];
        MoveDraw<T> md = move_draw<T>(seed, w, st, (uint32_t)e);
        const T n0 = md.n0, n1 = md.n1, n2 = md.n2;
        T nx, ny, nz, dlx = 0, dly = 0, dlz = 0;
        T logG = 0, R = 0, du;
        T un[SH::NE], u1n = 0;
        if (MOVE == MOVE_ONE_DRIFT) {
            // drift at the current position: grad ln D (from the current
            // inverse) + grad u; then the Langevin proposal
            MOEval<SH, T, SIG, 1, 0> mc;
            mc.run(S, rx, ry, rz);
            T ax = 0, ay = 0, az = 0;
#pragma unroll
            for (int k = 0; k < NS; ++k) { T d = DI(k, q); ax += mc.gx[k] * d; ay += mc.gy[k] * d; az += mc.gz[k] * d; }
            T g0[3], g1[3];
            jastrow_delta<SH, T, SIG, true>(S, P, e, rx, ry, rz, rx, ry, rz, g0, g1);
            T Fx = 2 * (ax + g0[0]), Fy = 2 * (ay + g0[1]), Fz = 2 * (az + g0[2]);
            dlx = tau * Fx; dly = tau * Fy; dlz = tau * Fz;
            T m = fsqrt(dlx * dlx + dly * dly + dlz * dlz);
            if (m > maxd) { T s = maxd / m; dlx *= s; dly *= s; dlz *= s; }
            T sd2 = fsqrt(2 * tau);
            nx = rx + dlx + sd2 * n0; ny = ry + dly + sd2 * n1; nz = rz + dlz + sd2 * n2;
            MOEval<SH, T, SIG, 1, 0> mn;
            mn.run(S, nx, ny, nz);
#pragma unroll
            for (int k = 0; k < NS; ++k) { R += mn.v[k] * DI(k, q); mv[k] = mn.v[k]; }
            T gn[3];
            du = jastrow_delta<SH, T, SIG, true>(S, P, e, rx, ry, rz, nx, ny, nz, g0, gn);
            T bx = 0, by = 0, bz = 0;
#pragma unroll
            for (int k = 0; k < NS; ++k) { T d = DI(k, q); bx += mn.gx[k] * d; by += mn.gy[k] * d; bz += mn.gz[k] * d; }
            T iR = R != T(0) ? T(1) / R : T(0);
            bx = tau * 2 * (bx * iR + gn[0]); by = tau * 2 * (by * iR + gn[1]); bz = tau * 2 * (bz * iR + gn[2]);
            T mb = fsqrt(bx * bx + by * by + bz * bz);
            if (mb > maxd) { T s = maxd / mb; bx *= s; by *= s; bz *= s; }
            T fx = nx - rx - dlx, fy = ny - ry - dly, fz = nz - rz - dlz;
            T qx = rx - nx - bx, qy = ry - ny - by, qz = rz - nz - bz;
            logG = ((fx * fx + fy * fy + fz * fz) - (qx * qx + qy * qy + qz * qz)) / (4 * tau);
        } else {
            nx = rx + step * n0; ny = ry + step * n1; nz = rz + step * n2;
            MOEval<SH, T, SIG, 0, 0> mn;
            mn.run(S, nx, ny, nz);
#pragma unroll
            for (int k = 0; k < NS; ++k) { R += mn.v[k] * DI(k, q); mv[k] = mn.v[k]; }
            if constexpr (PAIRS) {
                du = jastrow_delta_cached<SH, T, SIG, TPB>(S, P, pc, e, u1c[e], nx, ny, nz, un, u1n);
            } else {
                T g0[3], g1[3];
                du = jastrow_delta<SH, T, SIG, false>(S, P, e, rx, ry, rz, nx, ny, nz, g0, g1);
            }
        }
        T ratio = R * fexp(du);
        T prob = ratio * ratio;
        if (MOVE == MOVE_ONE_DRIFT) prob *= fexp(logG);
        if (prob != prob) flg |= FLAG_NONFINITE;
        // fixed-node rejection: a proposal that changes the sign of psi is refused
        if (md.uacc < prob && R != T(0) && !(fixed_node && R < T(0))) {
            P.set(e, nx, ny, nz);
            T iR = T(1) / R;
            T cq[NM];
#pragma unroll
            for (int k = 0; k < NS; ++k) cq[k] = DI(k, q) * iR;
#pragma unroll
            for (int j = 0; j < NS; ++j) {
                T tj = 0;
#pragma unroll
                for (int k = 0; k < NS; ++k) tj += mv[k] * DI(k, j);
#pragma unroll
                for (int k = 0; k < NS; ++k) DI(k, j) -= cq[k] * tj;
            }
#pragma unroll
            for (int k = 0; k < NS; ++k) DI(k, q) = cq[k];
            if constexpr (PAIRS) {
                pair_cache_store<SH, T, SIG, TPB>(pc, e, un);
                if (SH::JAS == JAS_PADE_EEN) u1c[e] = u1n;
            }
            if (R < 0) sgn = -sgn;
            ++acc;
        }
    }
#undef DI
}

// A global load, at the L2 when CG (state that another SM wrote during the same
// kernel: this SM's L1 may hold an older copy).
template <bool CG, class V>
__device__ __forceinline__ V ld_state(const V* p) {
    if constexpr (CG) return __ldcg(p);
    else return *p;
}

// n_sweeps single-electron sweeps of walker w, staged through the calling
// thread's shared-memory columns sp / sd; the accepted moves and status bits
// are added to acc_out / flg_out.
// a: the walker arrays, c: the sweep controls; both the same const SweepArgs<T>
// of kernel parameters, or the same block-shared const volatile one.
// jcache (chunked sweeps only): the walker's pair cache and one-body terms as
// the previous chunk left them, [slot][Wcap], read instead of recomputed when
// jc_load and written back when jc_store (recomputing them gives the same
// values: the same expressions on the same positions).
// CG (chunked sweeps): the inverse and the pair cache are already in the
// thread's shared-memory columns (copied by the calling warp) and are written
// back by it; the positions, sign and one-body terms are read at the L2 here.
template <class SH, class T, int MOVE, int TPB, bool CG = false, class A, class C>
__device__ __forceinline__ void sweep_walker(const SysT<SH, T>& S, T* sp, T* sd, A& a, C& c, int w,
                                             unsigned& acc_out, int& flg_out, T* jcache = nullptr,
                                             bool jc_load = false, bool jc_store = false) {
    constexpr int NPC = sweep_pairs<SH, MOVE>();
    constexpr int NM = SH::NMAX;
    const int t = threadIdx.x;
    const PosCols<T, TPB, SH::NE> P(sp, t);
#pragma unroll
    for (int e = 0; e < SH::NE; ++e)
        P.set(e, ld_state<CG>(&a.pos[(size_t)(3 * e) * a.Wcap + w]), ld_state<CG>(&a.pos[(size_t)(3 * e + 1) * a.Wcap + w]),
              ld_state<CG>(&a.pos[(size_t)(3 * e + 2) * a.Wcap + w]));
    if constexpr (!CG) {
#pragma unroll
        for (int i = 0; i < 2 * NM * NM; ++i) sd[i * TPB + t] = a.dinv[(size_t)i * a.Wcap + w];
    }
    T* pc = sd + 2 * NM * NM * TPB + t;
    // one-body terms of the electrons (thread-local; the pair cache fills the
    // shared-memory budget of a walker)
    T u1c[SH::NE];
    if constexpr (NPC > 0) {
        if (CG && jc_load) {
            if (SH::JAS == JAS_PADE_EEN) {
#pragma unroll
                for (int e = 0; e < SH::NE; ++e) u1c[e] = __ldcg(&jcache[(size_t)(NPC + e) * a.Wcap + w]);
            }
        } else {
            pair_cache_fill<SH, T, TPB>(S, P, pc);
            if (SH::JAS == JAS_PADE_EEN) {
#pragma unroll 1
                for (int e = 0; e < SH::NE; ++e)
                    u1c[e] = one_body_u(S, P(e, 0), P(e, 1), P(e, 2));
            }
        }
    }
    int sgn = ld_state<CG>(&a.sign[w]);
    unsigned acc = 0;
    int flg = 0;
    for (int it = 0; it < c.n_sweeps; ++it) {
        uint64_t st = c.step0 + (uint64_t)it;
        sweep_sector<SH, T, 0, MOVE, TPB>(S, sp, sd, pc, u1c, t, (uint32_t)w, st, c.seed, c.step, c.tau, c.maxd,
                                          c.fixed_node, sgn, acc, flg);
        sweep_sector<SH, T, 1, MOVE, TPB>(S, sp, sd, pc, u1c, t, (uint32_t)w, st, c.seed, c.step, c.tau, c.maxd,
                                          c.fixed_node, sgn, acc, flg);
    }
#pragma unroll
    for (int e = 0; e < SH::NE; ++e)
#pragma unroll
        for (int c = 0; c < 3; ++c) a.pos[(size_t)(3 * e + c) * a.Wcap + w] = P(e, c);
    if constexpr (!CG) {
#pragma unroll
        for (int i = 0; i < 2 * NM * NM; ++i) a.dinv[(size_t)i * a.Wcap + w] = sd[i * TPB + t];
    }
    a.sign[w] = sgn;
    if constexpr (NPC > 0) {
        if (CG && jc_store) {
            if (SH::JAS == JAS_PADE_EEN) {
#pragma unroll
                for (int e = 0; e < SH::NE; ++e) jcache[(size_t)(NPC + e) * a.Wcap + w] = u1c[e];
            }
        }
    }
    acc_out += acc;
    flg_out |= flg;
}

// Occupancy target: all walkers of the 65 536-walker workload resident in
// one wave (152 SMs x 8 blocks x 64 threads), i.e. <= 128 registers/thread.
template <class SH, class T, int MOVE, int TPB>
__global__ void __launch_bounds__(TPB, (sizeof(T) == 4 ? 512 : 256) / TPB) k_sweep_one(const __grid_constant__ SysT<SH, T> S, T* __restrict__ gpos,
                                                   T* __restrict__ gdinv, int* __restrict__ gsign, int W, int Wcap,
                                                   int n_sweeps, uint64_t step0, T step, T tau, T maxd,
                                                   uint64_t seed, unsigned long long* acc_out, int* flags,
                                                   int fixed_node) {
    extern __shared__ __align__(16) unsigned char smraw[];
    T* sp = reinterpret_cast<T*>(smraw);
    T* sd = sp + 3 * SH::NE * TPB;
    const int w = blockIdx.x * TPB + threadIdx.x;
    if (w >= W) return;
    // kernel parameters: the measured-fastest form of this kernel (block-shared
    // volatile arguments use fewer registers here but issue slower)
    const SweepArgs<T> a{gpos, gdinv, gsign, acc_out, flags, step0, seed, step, tau, maxd, W, Wcap, n_sweeps,
                         fixed_node};
    unsigned acc = 0;
    int flg = 0;
    sweep_walker<SH, T, MOVE, TPB>(S, sp, sd, a, a, w, acc, flg);
    if (acc) atomicAdd(acc_out, (unsigned long long)acc);
    if (flg) atomicOr(flags, flg);
}

// 16-byte global -> shared copy at the L2 (cp.async.cg), and its completion.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Rows r of a warp's 32 walker columns, global [r][Wcap] from walker g0 <->
// shared [r][TPB] from column c0: 16 bytes per lane, four rows per instruction.
template <int TPB>
__device__ __forceinline__ void warp_rows_in(float* sm, const float* gm, int rows, size_t Wcap, int lane) {
    const int q = 4 * (lane & 7);
    for (int r = lane >> 3; r < rows; r += 4) cp_async16(sm + (size_t)r * TPB + q, gm + (size_t)r * Wcap + q);
}
template <int TPB>
__device__ __forceinline__ void warp_rows_out(float* gm, const float* sm, int rows, size_t Wcap, int lane) {
    const int q = 4 * (lane & 7);
    for (int r = lane >> 3; r < rows; r += 4)
        *reinterpret_cast<float4*>(gm + (size_t)r * Wcap + q) = *reinterpret_cast<const float4*>(sm + (size_t)r * TPB + q);
}

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_gpu(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Upper bound on the polls of a chunk's wait (with a 256 ns back-off: about a
// second) before it gives up and raises FLAG_TIMEOUT.
constexpr unsigned CHUNK_WAIT_POLLS = 1u << 22;

// The same sweeps as k_sweep_one, as (32-walker group g, chunk c of CH sweeps)
// units taken in the order u = c G + g by persistent warps (warp p: units p,
// p + P, p + 2P, ...), with P a whole number of warps per SM sub-partition.
// A group's chunks move between warps, so every sub-partition carries the same
// share of the work, where one warp per group for the whole launch leaves the
// sub-partitions with 3 or 4 warps each.  A unit starts once the group's
// previous chunk is published (done[g] = c, a bounded wait that raises
// FLAG_TIMEOUT and goes on when it gives up), reads the group's walker state at
// the L2, writes it back and publishes done[g] = c + 1.  It is launched
// cooperatively, so every warp is resident; a unit waits only for a unit with
// a smaller index, so the waits end.  done[] is zero at the launch.
template <class SH, class T, int MOVE, int TPB>
__global__ void __launch_bounds__(TPB, (MOVE == MOVE_ONE_GAUSS ? 16 : 12) * 32 / TPB) k_sweep_chunks(
    const __grid_constant__ SysT<SH, T> S, T* __restrict__ gpos, T* __restrict__ gdinv, int* __restrict__ gsign, int W,
    int Wcap, int n_sweeps, int chunk, uint64_t step0, T step, T tau, T maxd, uint64_t seed,
    unsigned long long* acc_out, int* flags, int fixed_node, unsigned* __restrict__ done, T* __restrict__ jcache) {
    static_assert(std::is_same<T, float>::value, "the warp-row copies move 4-byte columns");
    extern __shared__ __align__(16) unsigned char smraw[];
    T* sp = reinterpret_cast<T*>(smraw);
    T* sd = sp + 3 * SH::NE * TPB;
    const int lane = threadIdx.x & 31;
    const int G = (W + 31) / 32, n_chunks = (n_sweeps + chunk - 1) / chunk;
    const long long P = (long long)gridDim.x * (TPB / 32);
    const long long U = (long long)G * n_chunks;
    for (long long u = (long long)blockIdx.x * (TPB / 32) + (threadIdx.x >> 5); u < U; u += P) {
        const int g = (int)(u % G), c = (int)(u / G);
        if (c > 0) {
            if (lane == 0) {
                unsigned polls = 0;
                while (ld_acquire_gpu(done + g) < (unsigned)c) {
                    if (++polls > CHUNK_WAIT_POLLS) { atomicOr(flags, FLAG_TIMEOUT); break; }
                    __nanosleep(256);
                }
            }
            __syncwarp();
        }
        const int w = g * 32 + lane;
        const int s0 = c * chunk, ns = min(chunk, n_sweeps - s0);
        // the group's inverses (and, after its first chunk, pair caches) as whole
        // rows of the warp's columns; the slots past W lie inside Wcap and
        // travel unchanged
        constexpr int NDI = 2 * SH::NMAX * SH::NMAX, NPC = sweep_pairs<SH, MOVE>();
        T* sdw = sd + (threadIdx.x - lane);
        warp_rows_in<TPB>(sdw, gdinv + (size_t)g * 32, NDI, (size_t)Wcap, lane);
        if (NPC > 0 && c > 0) warp_rows_in<TPB>(sdw + NDI * TPB, jcache + (size_t)g * 32, NPC, (size_t)Wcap, lane);
        cp_async_wait_all();
        __syncwarp();
        unsigned acc = 0;
        int flg = 0;
        if (w < W) {
            const SweepArgs<T> a{gpos, gdinv, gsign, acc_out, flags, step0 + (uint64_t)s0, seed, step, tau, maxd, W,
                                 Wcap, ns, fixed_node};
            sweep_walker<SH, T, MOVE, TPB, true>(S, sp, sd, a, a, w, acc, flg, jcache, c > 0, c + 1 < n_chunks);
        }
        __syncwarp();
        warp_rows_out<TPB>(gdinv + (size_t)g * 32, sdw, NDI, (size_t)Wcap, lane);
        if (NPC > 0 && c + 1 < n_chunks) warp_rows_out<TPB>(jcache + (size_t)g * 32, sdw + NDI * TPB, NPC, (size_t)Wcap, lane);
        acc = __reduce_add_sync(0xffffffffu, acc);
        flg = (int)__reduce_or_sync(0xffffffffu, (unsigned)flg);
        __syncwarp();                          // the lanes' state writes before lane 0's release
        if (lane == 0) {
            __threadfence();
            st_release_gpu(done + g, (unsigned)(c + 1));
            if (acc) atomicAdd(acc_out, (unsigned long long)acc);
            if (flg) atomicOr(flags, flg);
        }
    }
}

// Batched form: one block per (system, TPB-walker tile); the system table is
// staged into shared memory ahead of the walker columns.
template <class SH, class T, int MOVE, int TPB>
__global__ void __launch_bounds__(TPB, (sizeof(T) == 4 ? 512 : 256) / TPB) kb_sweep_one(
    const BatchTile* __restrict__ tiles, int ntiles, const BatchRec* __restrict__ recs,
    const BatchCtl* __restrict__ ctl) {
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ SweepArgs<T> args;
    SysT<SH, T>& S = *reinterpret_cast<SysT<SH, T>*>(smraw);
    T* sp = reinterpret_cast<T*>(smraw + batch_table_bytes<SH, T>());
    T* sd = sp + 3 * SH::NE * TPB;
    if ((int)blockIdx.x >= ntiles) return;
    const BatchTile tl = tiles[blockIdx.x];
    if (threadIdx.x == 0) args = sweep_args<T>(recs[tl.rec], *ctl);
    stage_table(&S, recs[tl.rec].tab_s);
    __syncthreads();
    const volatile SweepArgs<T>& a = args;
    const int w = tl.w0 + (int)threadIdx.x;
    unsigned acc = 0;
    int flg = 0;
    if (w < a.W) sweep_walker<SH, T, MOVE, TPB>(S, sp, sd, a, a, w, acc, flg);
    if (acc) atomicAdd(a.acc, (unsigned long long)acc);
    if (flg) atomicOr(a.flags, flg);
}

// Batched refresh + E_L (compute type TC) with one compensated partial per tile.
template <class SH, class TC, class TS, int TPB>
__global__ void __launch_bounds__(TPB) kb_measure(const BatchTile* __restrict__ tiles, int ntiles,
                                                  const BatchRec* __restrict__ recs, double* tile_partial) {
    __shared__ __align__(16) unsigned char sraw[batch_table_bytes<SH, TC>()];
    SysT<SH, TC>& S = *reinterpret_cast<SysT<SH, TC>*>(sraw);
    int t0, t1;
    batch_tile_range(ntiles, t0, t1);
    int cur = -1;
    for (int ti = t0; ti < t1; ++ti) {
        const BatchTile tl = tiles[ti];
        if (tl.rec != cur) {
            stage_table(&S, recs[tl.rec].tab_d);   // block_partial ended the previous tile with a barrier
            __syncthreads();
            cur = tl.rec;
        }
        const BatchRec& R = recs[tl.rec];
        const int w = tl.w0 + (int)threadIdx.x;
        MeasureOut none;
        double e_l = measure_walker<SH, TC, TS, 0>(S, (const TS*)R.pos, (TS*)R.dinv, R.logabs, R.sign, R.el, w,
                                                   w < R.W, R.Wcap, 1, none, 0, R.flags);
        block_partial<TPB>(e_l, tile_partial, ti);
    }
}

// All-electron Metropolis steps (src/sampling/vmc.rs:95-119): every step
// proposes all electrons, evaluates psi and E_L at the proposal from scratch,
// accepts with min(1, psi'^2/psi^2).  Per-step block partial sums of E_L
// (Neumaier pairs) are written to partial[step][block] when requested.
template <class SH, class T, int MOVE, int TPB>
__global__ void __launch_bounds__(TPB) k_step_all(const __grid_constant__ SysT<SH, T> S, T* __restrict__ gpos,
                                                  double* __restrict__ glog, int* __restrict__ gsign,
                                                  double* __restrict__ gel, int W, int Wcap, int n_steps,
                                                  uint64_t step0, T step, uint64_t seed,
                                                  unsigned long long* acc_out, double* partial, int nblk,
                                                  int* flags) {
    const int t = threadIdx.x;
    const int w = blockIdx.x * TPB + t;
    const bool act = w < W;
    T r[SH::NE][3];
#pragma unroll
    for (int e = 0; e < SH::NE; ++e)
#pragma unroll
        for (int c = 0; c < 3; ++c) r[e][c] = act ? gpos[(size_t)(3 * e + c) * Wcap + w] : T(e + 1) * T(0.37 + c);
    double lp = act ? glog[w] : 0.0;
    int sg = act ? gsign[w] : 1;
    double el = act ? gel[w] : 0.0;
    unsigned acc = 0;
    int flg = 0;
    auto nostore = [](int, int, int, T) {};
    for (int it = 0; it < n_steps; ++it) {
        uint64_t st = step0 + (uint64_t)it;
        T rn[SH::NE][3];
#pragma unroll
        for (int e = 0; e < SH::NE; ++e) {
            U4 x = rng_draw(seed, (uint32_t)w, st, (uint32_t)e, TAG_PROPOSE);
            if (MOVE == MOVE_ALL_GAUSS) {
                T n0, n1, n2, n3;
                bm(x.x, x.y, n0, n1);
                bm(x.z, x.w, n2, n3);
                rn[e][0] = r[e][0] + step * n0; rn[e][1] = r[e][1] + step * n1; rn[e][2] = r[e][2] + step * n2;
            } else {
                rn[e][0] = r[e][0] + step * (to_u01(x.x, T(0)) - T(0.5));
                rn[e][1] = r[e][1] + step * (to_u01(x.y, T(0)) - T(0.5));
                rn[e][2] = r[e][2] + step * (to_u01(x.z, T(0)) - T(0.5));
            }
        }
        FullEval<SH, T, 0> ev;
        evaluate_config<SH, T, 0>(S, rn, ev, false, nostore, (T*)nullptr);
        U4 a = rng_draw(seed, (uint32_t)w, st, 0, TAG_ACCEPT);
        double prob = exp(2.0 * (ev.logabs - lp));
        bool accept = act && ev.ok && (to_u01(a.x, 0.0) < prob);
        if (accept) {
#pragma unroll
            for (int e = 0; e < SH::NE; ++e)
#pragma unroll
                for (int c = 0; c < 3; ++c) r[e][c] = rn[e][c];
            lp = ev.logabs;
            sg = ev.sign;
            el = (double)ev.el;
            ++acc;
            if (!isfinite(el)) flg |= FLAG_NONFINITE;
        }
        if (partial) block_partial<TPB>(act ? el : 0.0, partial + (size_t)it * 2 * nblk, blockIdx.x);
    }
    if (act) {
#pragma unroll
        for (int e = 0; e < SH::NE; ++e)
#pragma unroll
            for (int c = 0; c < 3; ++c) gpos[(size_t)(3 * e + c) * Wcap + w] = r[e][c];
        glog[w] = lp;
        gsign[w] = sg;
        gel[w] = el;
        atomicAdd(acc_out, (unsigned long long)acc);
        if (flg) atomicOr(flags, flg);
    }
}

// ---------------------------------------------------------------------------
// Per-shape launchers (instantiated by QMC_DEFINE_SHAPE in qmc_shape_*.cu).
// ---------------------------------------------------------------------------
static inline int cuda_status(cudaError_t e) {
    if (e != cudaSuccess) {
        std::fprintf(stderr, "qmc_gb300: CUDA error %s\n", cudaGetErrorString(e));
        return 2;
    }
    return 0;
}

int launch_sum_partials(const double* partial, int nblk, int nrows, double* out, cudaStream_t st);

template <class SH>
struct ShapeOps {
    static int init(const HostSys& hs, DevWalkers& dw, uint64_t seed, cudaStream_t st) {
        SysT<SH, double> S;
        if (!fill_sys(hs, S)) return 7;
        int tpb = 128, nb = (dw.W + tpb - 1) / tpb;
        if (dw.prec == 0) k_init<SH, double><<<nb, tpb, 0, st>>>(S, (double*)dw.pos, dw.W, dw.Wcap, seed);
        else k_init<SH, float><<<nb, tpb, 0, st>>>(S, (float*)dw.pos, dw.W, dw.Wcap, seed);
        ++g_launch_count;
        return cuda_status(cudaGetLastError());
    }

    template <class TC, class TS, int NR, bool DEL = false>
    static int measure2(const HostSys& hs, DevWalkers& dw, bool write_state, const MeasureOut& out, cudaStream_t st) {
        SysT<SH, TC> S;
        if (!fill_sys(hs, S)) return 7;
        constexpr int TPB = 64;
        int nb = (dw.W + TPB - 1) / TPB;
        double* partial = nullptr;
        if (write_state && dw.partial && dw.partial_cap >= 2 * nb + 1) partial = dw.partial;
        k_measure<SH, TC, TS, TPB, NR, DEL><<<nb, TPB, 0, st>>>(S, (const TS*)dw.pos, (TS*)dw.dinv, dw.logabs, dw.sign,
                                                            dw.el, dw.W, dw.Wcap, write_state ? 1 : 0, out,
                                                            hs.n_params(), partial, dw.flags);
        ++g_launch_count;
        int rc = cuda_status(cudaGetLastError());
        if (rc || !partial) return rc;
        return launch_sum_partials(partial, nb, 1, dw.partial + dw.partial_cap - 1, st);
    }

    template <bool VALUES>
    static int measure_split(const HostSys& hs, DevWalkers& dw, bool write_state, cudaStream_t st) {
        SysT<SH, ff> S;
        if (!fill_sys(hs, S)) return 7;
        if (dw.W == 0) return 0;
        dim3 g1((dw.W + 127) / 128, SH::NE);
        k_rows<SH, float, VALUES><<<g1, 128, 0, st>>>(S, (const float*)dw.pos, dw.rows, dw.W, dw.Wcap);
        ++g_launch_count;
        int rc = cuda_status(cudaGetLastError());
        if (rc) return rc;
        constexpr int TPB = 64;
        const int nb = (dw.W + TPB - 1) / TPB;
        double* partial = nullptr;
        if (write_state && dw.partial && dw.partial_cap >= 2 * nb + 1) partial = dw.partial;
        if (VALUES) partial = nullptr;
        k_assemble<SH, float, TPB, VALUES><<<nb, TPB, 0, st>>>(S, dw.rows, (float*)dw.dinv, dw.logabs, dw.sign, dw.el,
                                                               dw.W, dw.Wcap, write_state ? 1 : 0, partial, dw.flags);
        ++g_launch_count;
        rc = cuda_status(cudaGetLastError());
        if (rc || !partial) return rc;
        return launch_sum_partials(partial, nb, 1, dw.partial + dw.partial_cap - 1, st);
    }

    static int measure(const HostSys& hs, DevWalkers& dw, int cp, bool ws, const MeasureOut& out, cudaStream_t st) {
        if (out.O) {
            if (SH::JAS != JAS_PADE_EEN || cp != 0 || dw.prec != 0) return 7;
            if (out.dEL) return measure2<double, double, SH::NROT, true>(hs, dw, ws, out, st);
            return measure2<double, double, SH::NROT>(hs, dw, ws, out, st);
        }
        if (cp == 0) {
            if (dw.prec == 0) return measure2<double, double, 0>(hs, dw, ws, out, st);
            // FP64-class refresh on the FP32 pipe: the two-pass form when only
            // the walker state is wanted, else the single-kernel form
            if (dw.rows && !out.grad && !out.lap && !out.fhf && !out.omega)
                return out.inverse_only ? measure_split<true>(hs, dw, ws, st) : measure_split<false>(hs, dw, ws, st);
            return measure2<ff, float, 0>(hs, dw, ws, out, st);
        }
        if (dw.prec == 1) return measure2<float, float, 0>(hs, dw, ws, out, st);
        return 7;
    }

    template <class T, int MOVE>
    static int sweep_one(const HostSys& hs, DevWalkers& dw, int n, uint64_t s0, double step, double tau, double maxd,
                         uint64_t seed, cudaStream_t st) {
        SysT<SH, T> S;
        if (!fill_sys(hs, S)) return 7;
        constexpr int TPB = 64;
        size_t smem = sizeof(T) * TPB * sweep_words<SH, MOVE>();
        auto kern = k_sweep_one<SH, T, MOVE, TPB>;
        static bool attr_set = false;
        if (!attr_set) {
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
            attr_set = true;
        }
        if constexpr (std::is_same<T, float>::value) {
            int rc = 0;
            if (sweep_chunks<T, MOVE>(S, dw, n, s0, step, tau, maxd, seed, smem, st, rc)) return rc;
        }
        int nb = (dw.W + TPB - 1) / TPB;
        kern<<<nb, TPB, smem, st>>>(S, (T*)dw.pos, (T*)dw.dinv, dw.sign, dw.W, dw.Wcap, n, s0, (T)step, (T)tau,
                                    (T)maxd, seed, dw.acc, dw.flags, dw.fixed_node);
        ++g_launch_count;
        return cuda_status(cudaGetLastError());
    }

    // The chunked form of sweep_one (k_sweep_chunks) when the set fills every SM
    // sub-partition with CHUNK_WARPS warps at least once and the stream is not
    // being captured; false leaves the launch to the one-warp-per-group kernel.
    static constexpr int CHUNK_SWEEPS = 8, CHUNK_WARPS = 3;
    template <class T, int MOVE>
    static bool sweep_chunks(const SysT<SH, T>& S, DevWalkers& dw, int n, uint64_t s0, double step, double tau,
                             double maxd, uint64_t seed, size_t smem, cudaStream_t st, int& rc) {
        constexpr int TPB = 64, BPS = 4 * CHUNK_WARPS * 32 / TPB;   // blocks per SM
        static int nsm = 0;
        if (!nsm) {
            int dev = 0;
            if (cudaGetDevice(&dev) != cudaSuccess ||
                cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
                return false;
        }
        const int G = (dw.W + 31) / 32;
        if (!dw.chunk_done || n < 2 * CHUNK_SWEEPS || G < nsm * BPS * (TPB / 32)) return false;
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return false;
        auto kern = k_sweep_chunks<SH, T, MOVE, TPB>;
        static int occ = -1;
        if (occ < 0) {
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, TPB, smem) != cudaSuccess) occ = 0;
        }
        if (occ < BPS) return false;
        constexpr int NJC = sweep_pairs<SH, MOVE>() > 0 ? sweep_pairs<SH, MOVE>() + SH::NE : 0;
        if (NJC > 0 && !dw.chunk_jc) {
            if (cudaMalloc((void**)&dw.chunk_jc, sizeof(float) * NJC * (size_t)dw.Wcap) != cudaSuccess) {
                dw.chunk_jc = nullptr;
                return false;
            }
        }
        rc = cuda_status(cudaMemsetAsync(dw.chunk_done, 0, 4 * (size_t)G, st));
        if (rc) return true;
        T* pos = (T*)dw.pos;
        T* dinv = (T*)dw.dinv;
        int* sign = dw.sign;
        int W = dw.W, Wcap = dw.Wcap, ns = n, ch = CHUNK_SWEEPS, fixed = dw.fixed_node;
        T stp = (T)step, ta = (T)tau, md = (T)maxd;
        uint64_t step0 = s0, sd = seed;
        unsigned long long* acc = dw.acc;
        int* flags = dw.flags;
        unsigned* done = dw.chunk_done;
        T* jc = (T*)dw.chunk_jc;
        void* args[] = {(void*)&S, &pos,   &dinv, &sign,  &W,   &Wcap, &ns,    &ch,    &step0,
                        &stp,      &ta,    &md,   &sd,    &acc, &flags, &fixed, &done, &jc};
        rc = cuda_status(cudaLaunchCooperativeKernel((const void*)kern, dim3(nsm * BPS), dim3(TPB), args, smem, st));
        ++g_launch_count;
        return true;
    }

    template <class T, int MOVE>
    static int step_all(const HostSys& hs, DevWalkers& dw, int n, uint64_t s0, double step, uint64_t seed,
                        cudaStream_t st, double* partial) {
        SysT<SH, T> S;
        if (!fill_sys(hs, S)) return 7;
        constexpr int TPB = 64;
        int nb = (dw.W + TPB - 1) / TPB;
        k_step_all<SH, T, MOVE, TPB><<<nb, TPB, 0, st>>>(S, (T*)dw.pos, dw.logabs, dw.sign, dw.el, dw.W, dw.Wcap, n,
                                                          s0, (T)step, seed, dw.acc, partial, nb, dw.flags);
        ++g_launch_count;
        return cuda_status(cudaGetLastError());
    }

    // ---- batched launches ---------------------------------------------------
    static constexpr int BTPB = 64;

    // Device copy of the system table (slot 0 FP64, slot 1 FP32), cached in
    // the HostSys and rebuilt when its parameters or nuclei change.
    template <class T>
    static int table(const HostSys& hs, const SysT<SH, T>** out) {
        const int slot = std::is_same<T, double>::value ? 0 : (std::is_same<T, float>::value ? 1 : 2);
        if (!hs.dev_table[slot] || hs.dev_table_version[slot] != hs.version) {
            SysT<SH, T> h;
            if (!fill_sys(hs, h)) return 7;
            if (!hs.dev_table[slot] && cudaMalloc(&hs.dev_table[slot], sizeof(h)) != cudaSuccess) return 8;
            if (cudaMemcpy(hs.dev_table[slot], &h, sizeof(h), cudaMemcpyHostToDevice) != cudaSuccess) return 2;
            hs.dev_table_version[slot] = hs.version;
        }
        *out = static_cast<const SysT<SH, T>*>(hs.dev_table[slot]);
        return 0;
    }

    // tab_s: the sweep table (walker precision); tab_d: the refresh table
    // (FP64 for FP64 walkers, float-float for FP32 walkers).
    static int batch_tables(const HostSys& hs, int prec, BatchRec& r) {
        r.ktab = nullptr;
        if (prec == 0) {
            const SysT<SH, double>* d;
            int rc = table<double>(hs, &d);
            if (rc) return rc;
            r.tab_d = r.tab_s = d;
            return 0;
        }
        const SysT<SH, ff>* m;
        const SysT<SH, float>* f;
        int rc = table<ff>(hs, &m);
        if (!rc) rc = table<float>(hs, &f);
        if (rc) return rc;
        r.tab_d = m;
        r.tab_s = f;
        return 0;
    }

    template <class T, int MOVE>
    static size_t batch_sweep_smem() {
        return batch_table_bytes<SH, T>() + sizeof(T) * BTPB * sweep_words<SH, MOVE>();
    }

    template <class T, int MOVE>
    static int batch_sweep_t(const BatchClass& bc, const BatchCtl* ctl, cudaStream_t st, int* occ) {
        const size_t smem = batch_sweep_smem<T, MOVE>();
        auto kern = kb_sweep_one<SH, T, MOVE, BTPB>;
        static bool attr = false;
        if (!attr) {
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            attr = true;
        }
        if (occ) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, kern, BTPB, smem) == cudaSuccess ? 0 : 2;
        if (bc.ntiles == 0) return 0;
        kern<<<bc.ntiles, BTPB, smem, st>>>(bc.tiles, bc.ntiles, bc.recs, ctl);
        ++g_launch_count;
        return cuda_status(cudaGetLastError());
    }

    // occ != nullptr: report resident blocks per SM instead of launching.
    static int batch_sweep(const BatchClass& bc, int mk, const BatchCtl* ctl, cudaStream_t st, int* occ = nullptr) {
        if (mk == MOVE_ONE_GAUSS)
            return bc.prec == 0 ? batch_sweep_t<double, MOVE_ONE_GAUSS>(bc, ctl, st, occ)
                                : batch_sweep_t<float, MOVE_ONE_GAUSS>(bc, ctl, st, occ);
        if (mk == MOVE_ONE_DRIFT)
            return bc.prec == 0 ? batch_sweep_t<double, MOVE_ONE_DRIFT>(bc, ctl, st, occ)
                                : batch_sweep_t<float, MOVE_ONE_DRIFT>(bc, ctl, st, occ);
        return 7;
    }

    template <class TC, class TS>
    static int batch_measure_t(const BatchClass& bc, cudaStream_t st, int* occ) {
        auto kern = kb_measure<SH, TC, TS, BTPB>;
        if (occ) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, kern, BTPB, 0) == cudaSuccess ? 0 : 2;
        if (bc.ntiles == 0) return 0;
        const int grid =
            bc.grid_measure > 0 ? (bc.grid_measure < bc.ntiles ? bc.grid_measure : bc.ntiles) : bc.ntiles;
        kern<<<grid, BTPB, 0, st>>>(bc.tiles, bc.ntiles, bc.recs, bc.tile_partial);
        ++g_launch_count;
        return cuda_status(cudaGetLastError());
    }

    // FP32 walkers: the two-pass float-float refresh (rows, then assembly).
    static int batch_measure_split(const BatchClass& bc, cudaStream_t st, int* occ) {
        auto k1 = kb_rows<SH, float, BTPB>;
        auto k2 = kb_assemble<SH, float, BTPB>;
        static int occ1 = 0, nsm = 0;
        if (!occ1) {
            int dev = 0;
            cudaGetDevice(&dev);
            if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 2;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ1, k1, BTPB, 0) != cudaSuccess) return 2;
            if (occ1 < 1) occ1 = 1;
        }
        if (occ) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, k2, BTPB, 0) == cudaSuccess ? 0 : 2;
        if (bc.ntiles == 0) return 0;
        const int items = bc.ntiles * SH::NE;
        const int g1 = occ1 * nsm < items ? occ1 * nsm : items;
        k1<<<g1, BTPB, 0, st>>>(bc.tiles, bc.ntiles, bc.recs);
        ++g_launch_count;
        int rc = cuda_status(cudaGetLastError());
        if (rc) return rc;
        const int g2 =
            bc.grid_measure > 0 ? (bc.grid_measure < bc.ntiles ? bc.grid_measure : bc.ntiles) : bc.ntiles;
        k2<<<g2, BTPB, 0, st>>>(bc.tiles, bc.ntiles, bc.recs, bc.tile_partial);
        ++g_launch_count;
        return cuda_status(cudaGetLastError());
    }

    static int batch_measure(const BatchClass& bc, cudaStream_t st, int* occ = nullptr) {
        return bc.prec == 0 ? batch_measure_t<double, double>(bc, st, occ) : batch_measure_split(bc, st, occ);
    }

    template <bool ALL>
    static int sweep_part(const HostSys& hs, DevWalkers& dw, int mk, int n, uint64_t s0, double step, double tau,
                          double maxd, uint64_t seed, cudaStream_t st, double* partial) {
        bool all = (mk == MOVE_ALL_GAUSS || mk == MOVE_ALL_BOX);
        if (all != ALL) return 1;
        if (ALL) {
            if (dw.prec == 0) return mk == MOVE_ALL_BOX ? step_all<double, MOVE_ALL_BOX>(hs, dw, n, s0, step, seed, st, partial)
                                                        : step_all<double, MOVE_ALL_GAUSS>(hs, dw, n, s0, step, seed, st, partial);
            return mk == MOVE_ALL_BOX ? step_all<float, MOVE_ALL_BOX>(hs, dw, n, s0, step, seed, st, partial)
                                      : step_all<float, MOVE_ALL_GAUSS>(hs, dw, n, s0, step, seed, st, partial);
        }
        if (dw.prec == 0) return mk == MOVE_ONE_DRIFT ? sweep_one<double, MOVE_ONE_DRIFT>(hs, dw, n, s0, step, tau, maxd, seed, st)
                                                      : sweep_one<double, MOVE_ONE_GAUSS>(hs, dw, n, s0, step, tau, maxd, seed, st);
        return mk == MOVE_ONE_DRIFT ? sweep_one<float, MOVE_ONE_DRIFT>(hs, dw, n, s0, step, tau, maxd, seed, st)
                                    : sweep_one<float, MOVE_ONE_GAUSS>(hs, dw, n, s0, step, tau, maxd, seed, st);
    }
};

#define QMC_DEFINE_SHAPE_MEASURE(NAME, SHAPE)                                                                  \
    int shape_init_##NAME(const HostSys& hs, DevWalkers& dw, uint64_t seed, cudaStream_t st) {               \
        return ShapeOps<SHAPE>::init(hs, dw, seed, st);                                                       \
    }                                                                                                         \
    int shape_measure_##NAME(const HostSys& hs, DevWalkers& dw, int cp, bool ws, const MeasureOut& out,       \
                             cudaStream_t st) {                                                               \
        return ShapeOps<SHAPE>::measure(hs, dw, cp, ws, out, st);                                             \
    }                                                                                                         \
    int shape_nmax_##NAME() { return SHAPE::NMAX; }

#define QMC_DEFINE_SHAPE_ONE(NAME, SHAPE)                                                                      \
    int shape_sweep_one_##NAME(const HostSys& hs, DevWalkers& dw, int mk, int n, uint64_t s0, double step,   \
                               double tau, double maxd, uint64_t seed, cudaStream_t st) {                     \
        return ShapeOps<SHAPE>::template sweep_part<false>(hs, dw, mk, n, s0, step, tau, maxd, seed, st, nullptr);                 \
    }

#define QMC_DEFINE_SHAPE_BATCH_SWEEP(NAME, SHAPE)                                                              \
    int shape_batch_sweep_##NAME(const BatchClass& bc, int mk, const BatchCtl* ctl, cudaStream_t st, int* occ) { \
        return ShapeOps<SHAPE>::batch_sweep(bc, mk, ctl, st, occ);                                            \
    }

#define QMC_DEFINE_SHAPE_BATCH_MEASURE(NAME, SHAPE)                                                            \
    int shape_batch_measure_##NAME(const BatchClass& bc, cudaStream_t st, int* occ) {                         \
        return ShapeOps<SHAPE>::batch_measure(bc, st, occ);                                                   \
    }                                                                                                         \
    int shape_batch_tables_##NAME(const HostSys& hs, int prec, BatchRec& r) {                                 \
        return ShapeOps<SHAPE>::batch_tables(hs, prec, r);                                                    \
    }                                                                                                         \
    int shape_batch_width_##NAME() { return ShapeOps<SHAPE>::BTPB; }

#define QMC_DEFINE_SHAPE_ALL(NAME, SHAPE)                                                                      \
    int shape_step_all_##NAME(const HostSys& hs, DevWalkers& dw, int mk, int n, uint64_t s0, double step,    \
                              uint64_t seed, cudaStream_t st, double* partial) {                              \
        return ShapeOps<SHAPE>::template sweep_part<true>(hs, dw, mk, n, s0, step, 0.0, 0.0, seed, st, partial);                  \
    }

}  // namespace qmc

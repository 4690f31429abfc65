// qmc_jastrow3_logderiv.h -- parameter log-derivatives of the Jastrow3 factor
// for one configuration, compiled for the device (k_jastrow3_logderiv) and,
// unchanged, for the host checks of this header.
//
// u = sum_{i<j} a_s r_ij / (1 + b_s r_ij) - sum_{i,I} A_t Z_I r_iI / (1 + B_t r_iI)
// (src/correlation/jastrow.rs:138-449) with a and b per spin class s
// (antiparallel, parallel) and A and B per nuclear species t; ln J = u, so
//   d u / d b_s = -a_s r^2 / (1 + b_s r)^2,   d u / d a_s = r / (1 + b_s r),
//   d u / d B_t = A_t Z r^2 / (1 + B_t r)^2,  d u / d A_t = -Z r / (1 + B_t r),
// summed over the pairs of each class (jastrow.rs:326-391 ties the classes:
// its four derivatives are sums of these eight).
#pragma once
#include <cmath>

#ifndef QMC_JHD
#if defined(__CUDACC__)
#define QMC_JHD __host__ __device__
#else
#define QMC_JHD
#endif
#endif

namespace qmc {

// p = [b_anti, b_para, a_anti, a_para, B_0, B_1, A_0, A_1]; electrons
// 0 .. n_up-1 are spin up, the rest spin down; pos(i, c) is coordinate c of
// electron i; nuc = [n_nuc][5] (x, y, z, Z, species 0 or 1).  O receives the
// eight derivatives in the order of p.
template <class Pos>
QMC_JHD inline void jastrow3_log_derivatives(int N, int n_up, int n_nuc, const double* nuc, const double* p,
                                             const Pos& pos, double* O) {
    double db_anti = 0.0, db_para = 0.0, da_anti = 0.0, da_para = 0.0;
    double dB0 = 0.0, dB1 = 0.0, dA0 = 0.0, dA1 = 0.0;
    for (int i = 0; i < N; ++i) {
        const double xi = pos(i, 0), yi = pos(i, 1), zi = pos(i, 2);
        const bool up_i = i < n_up;
        for (int j = i + 1; j < N; ++j) {
            const double dx = xi - pos(j, 0), dy = yi - pos(j, 1), dz = zi - pos(j, 2);
            const double d = sqrt(dx * dx + dy * dy + dz * dz);
            if (up_i == (j < n_up)) {
                const double den = 1.0 + p[1] * d;
                db_para += -p[3] * d * d / (den * den);
                da_para += d / den;
            } else {
                const double den = 1.0 + p[0] * d;
                db_anti += -p[2] * d * d / (den * den);
                da_anti += d / den;
            }
        }
        for (int I = 0; I < n_nuc; ++I) {
            const double* n = nuc + 5 * I;
            const double dx = xi - n[0], dy = yi - n[1], dz = zi - n[2];
            const double d = sqrt(dx * dx + dy * dy + dz * dz);
            const double Zi = n[3];
            if (n[4] == 0.0) {
                const double den = 1.0 + p[4] * d;
                dB0 += p[6] * Zi * d * d / (den * den);
                dA0 += -Zi * d / den;
            } else {
                const double den = 1.0 + p[5] * d;
                dB1 += p[7] * Zi * d * d / (den * den);
                dA1 += -Zi * d / den;
            }
        }
    }
    O[0] = db_anti; O[1] = db_para; O[2] = da_anti; O[3] = da_para;
    O[4] = dB0; O[5] = dB1; O[6] = dA0; O[7] = dA1;
}

// Jastrow-parameter part of dE_L / dp for one configuration, given G_i =
// grad_i ln|psi| (all factors) per electron: E_L = -1/2 sum_i (l_i + 2 g_i.j_i
// + lu_i + |j_i|^2) + V, with j_i, lu_i the Jastrow gradient and Laplacian,
// so dE_L/dp = -1/2 sum_i [ d lu_i/dp + 2 G_i . d j_i/dp ].  Per e-e pair of
// class s with den = 1 + b_s r (j_i gains f r_ij, j_j loses it, lu_i and lu_j
// both gain l):
//   d/da_s: f = 1/(den^2 r),  l = 2/(r den^2) - 2 b_s/den^3
//   d/db_s: f = -2 a_s/den^3, l = -6 a_s/den^4
// per e-n pair with den = 1 + B_t r and j_i gaining f r_iI, lu_i gaining l:
//   d/dA_t: f = -Z/(den^2 r), l = -2 Z/(r den^2) + 2 Z B_t/den^3
//   d/dB_t: f = 2 A_t Z/den^3, l = 6 A_t Z/den^4
// (pairs closer than 1e-10 are skipped, as the Jastrow itself skips them,
// src/correlation/jastrow.rs:256,277).  grad(i, c) is component c of G_i;
// dE receives the eight derivatives in the order of p.
template <class Pos, class Grad>
QMC_JHD inline void jastrow3_el_derivatives(int N, int n_up, int n_nuc, const double* nuc, const double* p,
                                            const Pos& pos, const Grad& grad, double* dE) {
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = 0; i < N; ++i) {
        const double xi = pos(i, 0), yi = pos(i, 1), zi = pos(i, 2);
        const double gxi = grad(i, 0), gyi = grad(i, 1), gzi = grad(i, 2);
        const bool up_i = i < n_up;
        for (int j = i + 1; j < N; ++j) {
            const double dx = xi - pos(j, 0), dy = yi - pos(j, 1), dz = zi - pos(j, 2);
            const double d = sqrt(dx * dx + dy * dy + dz * dz);
            if (d < 1e-10) continue;
            const int c = (up_i == (j < n_up)) ? 1 : 0;
            const double a = p[2 + c], b = p[c];
            const double den = 1.0 + b * d, i1 = 1.0 / den, i2 = i1 * i1, i3 = i2 * i1;
            const double gdot = (gxi - grad(j, 0)) * dx + (gyi - grad(j, 1)) * dy + (gzi - grad(j, 2)) * dz;
            const double fa = i2 / d, la = 2.0 * i2 / d - 2.0 * b * i3;
            const double fb = -2.0 * a * i3, lb = -6.0 * a * i3 * i1;
            acc[2 + c] += 2.0 * la + 2.0 * fa * gdot;
            acc[c] += 2.0 * lb + 2.0 * fb * gdot;
        }
        for (int I = 0; I < n_nuc; ++I) {
            const double* n = nuc + 5 * I;
            const double dx = xi - n[0], dy = yi - n[1], dz = zi - n[2];
            const double d = sqrt(dx * dx + dy * dy + dz * dz);
            if (d < 1e-10) continue;
            const int t = n[4] == 0.0 ? 0 : 1;
            const double Zi = n[3], A = p[6 + t] * Zi, B = p[4 + t];
            const double den = 1.0 + B * d, i1 = 1.0 / den, i2 = i1 * i1, i3 = i2 * i1;
            const double gdot = gxi * dx + gyi * dy + gzi * dz;
            const double fA = -Zi * i2 / d, lA = -2.0 * Zi * i2 / d + 2.0 * Zi * B * i3;
            const double fB = 2.0 * A * i3, lB = 6.0 * A * i3 * i1;
            acc[6 + t] += lA + 2.0 * fA * gdot;
            acc[4 + t] += lB + 2.0 * fB * gdot;
        }
    }
    for (int k = 0; k < 8; ++k) dE[k] = -0.5 * acc[k];
}

}  // namespace qmc

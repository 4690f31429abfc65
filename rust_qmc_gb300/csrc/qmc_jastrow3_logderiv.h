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

}  // namespace qmc

// qmc_roofline.cpp -- algorithmic operation and byte counts of the walker
// kernels, per system: the denominators of the benchmark's roofline figures.
// One formula per kernel family, written once here so that the benchmark
// and the documentation quote the same counts.
#include <algorithm>
#include <cmath>
#include "qmc_internal.h"

namespace qmc {

namespace {

// Reciprocal vectors of the electron-gas Ewald sum: the half space of
// integer vectors with |n| <= K (or the cube |n_i| <= K in the reference's form).
int count_kvectors(int K, bool cube) {
    int nk = 0;
    for (int nx = 0; nx <= K; ++nx)
        for (int ny = -K; ny <= K; ++ny)
            for (int nz = -K; nz <= K; ++nz) {
                if (nx == 0 && (ny < 0 || (ny == 0 && nz <= 0))) continue;
                if (!cube && nx * nx + ny * ny + nz * nz > K * K) continue;
                ++nk;
            }
    return nk;
}

}  // namespace

// out: [0] sweep FP32 operations per single-electron Gaussian proposal
//      (transcendentals count one), [1] walker state bytes read and written by
//      one sweep launch, per walker, [2] refresh operations per walker
//      (FP64-class), [3] refresh HBM bytes per walker.
void roofline_counts(const HostSys& hs, int prec, double acc, double out[4]) {
    const double N = hs.N, Nn = hs.n_nuc, nu = hs.n_up, nd = hs.n_dn;
    // electron-weighted sector sizes: a move of an up electron costs n_up-sized work
    const double n1 = (nu * nu + nd * nd) / N, n2 = (nu * nu * nu + nd * nd * nd) / N;
    int n_prim = 0;
    for (const HostShell& s : hs.shells) n_prim += (int)s.exps.size();
    const double ts = prec == 0 ? 8.0 : 4.0;
    const double dinv = (double)dinv_elems_of_shape(hs.shape);
    out[1] = 2.0 * ((3.0 * N + dinv) * ts + 4.0);
    double rows = prec == 1 ? 2.0 * (double)refresh_rows_bytes(hs.shape) : 0.0;
    out[3] = 3.0 * N * ts + dinv * ts + 20.0 + rows;
    if (hs.basis == 2) {
        // plane waves: per proposal 3 FMA + sincos per orbital, complex ratio,
        // Jastrow old and new over N-1 partners (minimum image), complex
        // Sherman-Morrison on acceptance
        out[0] = 30.0 + 12.0 * n1 + 27.0 * (N - 1.0) + acc * (16.0 * n2 + 4.0 * n1);
        const bool cube = (hs.quirks & 4) != 0;
        const int K = cube ? 7 : (int)hs.jas[5];
        const double nk = count_kvectors(K, cube);
        const double pairs = N * (N - 1.0) / 2.0;
        out[2] = N * 5.0 * n1                               // orbital phases
                 + 16.0 * (nu * nu * nu + nd * nd * nd)         // complex Gauss-Jordan on [D | I]
                 + 20.0 * N * (N - 1.0)                       // Jastrow from both ends
                 + pairs * (20.0 + (cube ? 0.0 : 26.0 * 12.0))  // real-space Ewald (minimum image + images)
                 + nk * (8.0 * N + 10.0);                      // reciprocal sum
    } else {
        const double en = hs.jk == 2 ? Nn : 0.0;              // electron-nucleus Jastrow terms
        out[0] = 30.0 + 8.0 * Nn + 5.0 * n_prim + 2.0 * hs.n_ao * n1 + 2.0 * n1 +
                 24.0 * (N - 1.0 + en) + acc * (4.0 * n2 + n1);
        const double pairs = N * (N - 1.0) / 2.0;
        out[2] = N * (8.0 * Nn + 9.0 * n_prim)                // AO values, gradients, Laplacians
                 + N * 10.0 * hs.n_ao * n1                    // MO contraction of 5 quantities
                 + 4.0 * (nu * nu * nu + nd * nd * nd)          // Gauss-Jordan on [D | I]
                 + 8.0 * (nu * nu + nd * nd)                    // kinetic contractions
                 + 20.0 * pairs + 20.0 * N * en;               // Jastrow + Coulomb
    }
}

}  // namespace qmc

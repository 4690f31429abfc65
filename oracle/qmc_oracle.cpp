// qmc_oracle.cpp -- FP64 CPU restatement of rust_qmc's walker-ensemble path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the correctness oracle and the timed
// CPU baseline.  Nothing in the product (the rust_qmc_gb300 package and its
// CUDA library) may link, load or call it; only tests/, the smoke check and
// the bench's CPU-baseline leg do.
//
// Parity pinning: the reference (a Rust crate) cannot be built here (no
// cargo/rustc), so this restatement is pinned against the reference's own
// golden scalars (src/lib.rs:31-56: Jastrow1 value 0.7788007831 and gradient
// -/+0.09735009789), its finite-difference self-consistency tests
// (src/lib.rs:88-267, src/systems/methane.rs:1310-1373,
// src/systems/benzene.rs:954-1006), its range checks (V_nn windows,
// geometry), and the published Philox4x32-10 known-answer vectors.
//
// Structure follows the reference literally where it matters for the timed
// baseline: every evaluate() rebuilds each spin sector's Slater matrix by
// evaluating every AO once per MO (src/systems/methane.rs:781-787,812-831)
// and factorises it from scratch.  The one deliberate change is that psi is
// carried as (log|psi|, sign) so that benzene-size products do not underflow;
// gradients and Laplacians are returned divided by psi, which is the
// reference's expression divided by psi.
//
// Reference crates that are not in the mount are restated: nalgebra 0.33.0's
// determinant/try_inverse (LU with partial pivoting), rand 0.8.5's thread_rng
// is replaced by counter-based Philox4x32-10 (Salmon et al., SC'11) so that
// trajectories are reproducible.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <thread>
#include <algorithm>
#include <complex>

extern "C" {

// Same field order as qmc_system_desc in include/qmc.h (the tests check the
// layouts agree).  Kept as an independent declaration: the oracle does not
// include product headers.
typedef struct {
    int n_elec;
    const int* spins;            // [n_elec] +1 / -1, reference electron order
    int n_nuc;
    const double* nuc_pos;       // [n_nuc*3]
    const double* nuc_charge;    // [n_nuc]
    const int* nuc_species;      // [n_nuc] one-body Jastrow species (0/1) or NULL
    int basis_kind;              // 0 = contracted Gaussian, 1 = Slater-type
    int n_ao;
    const int* ao_nuc;           // [n_ao]
    const int* ao_l;             // [n_ao]
    const int* ao_m;             // [n_ao]
    const int* ao_prim_off;      // [n_ao+1]
    const double* prim_exp;
    const double* prim_coef;
    const int* prim_pow;         // Slater-type radial powers (NULL for Gaussians)
    int n_mo;
    const double* mo_coef;       // [n_mo*n_ao], row = MO
    const int* occ;              // [n_elec] MO that forms electron e's column
    int jastrow_kind;            // 0 none, 1 Pade-F (Jastrow1/2), 2 e-e + e-n Pade (Jastrow3)
    double jas_F;
    double jas[8];               // b_anti b_para a_anti a_para B0 B1 A0 A1
    int n_rot;
    const int* rot_occ;          // [n_rot]
    const int* rot_virt;         // [n_rot]
    const double* rot_angle;     // [n_rot]
    int quirks;                  // bit0 Jastrow2 gradient prefactor, bit1 Jastrow2 Laplacian
    const int* init_nuc;         // [n_elec] or NULL (origin)
    double init_sigma;
    double box_L;                // reserved for periodic systems (0 = open)
    int reserved[4];
} orc_system_desc;

}  // extern "C"

namespace {

struct V3 { double x, y, z; };
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double norm(V3 a) { return std::sqrt(dot(a, a)); }
inline double comp(V3 a, int m) { return m == 0 ? a.x : (m == 1 ? a.y : a.z); }
inline void add_comp(V3& a, int m, double v) { if (m == 0) a.x += v; else if (m == 1) a.y += v; else a.z += v; }

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC'11).  Multipliers and Weyl key increments from the paper.
// ---------------------------------------------------------------------------
struct U4 { uint32_t v[4]; };
U4 philox(U4 c, uint32_t k0, uint32_t k1) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
    for (int r = 0; r < 10; ++r) {
        if (r) { k0 += W0; k1 += W1; }
        uint64_t p0 = (uint64_t)M0 * c.v[0];
        uint64_t p1 = (uint64_t)M1 * c.v[2];
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        U4 n;
        n.v[0] = hi1 ^ c.v[1] ^ k0;
        n.v[1] = lo1;
        n.v[2] = hi0 ^ c.v[3] ^ k1;
        n.v[3] = lo0;
        c = n;
    }
    return c;
}

// Counter layout shared with the CUDA kernels (documented in include/qmc.h):
// c0 = walker id, c1 = step (low 32 bits), c2 = electron / sub-index,
// c3 = tag | (step high 16 bits << 16).
enum { TAG_PROPOSE = 1, TAG_ACCEPT = 2, TAG_INIT = 3, TAG_BRANCH = 4 };
U4 draw(uint64_t seed, uint32_t walker, uint64_t step, uint32_t sub, uint32_t tag) {
    U4 c;
    c.v[0] = walker;
    c.v[1] = (uint32_t)step;
    c.v[2] = sub;
    c.v[3] = tag | ((uint32_t)((step >> 32) & 0xFFFFu) << 16);
    return philox(c, (uint32_t)seed, (uint32_t)(seed >> 32));
}
inline double u01(uint32_t x) { return ((double)x + 0.5) * (1.0 / 4294967296.0); }
inline double u24(uint32_t x) { return ((double)x + 0.5) * (1.0 / 16777216.0); }
// Box-Muller (Box & Muller 1958): two uniforms -> two standard normals.
inline void box_muller(uint32_t a, uint32_t b, double& n0, double& n1) {
    double r = std::sqrt(-2.0 * std::log(u01(a)));
    double t = 6.283185307179586476925286766559 * u01(b);
    n0 = r * std::cos(t);
    n1 = r * std::sin(t);
}

// ---------------------------------------------------------------------------
// System, built from the flat descriptor.
// ---------------------------------------------------------------------------
struct AO { int nuc, l, m, p0, p1; };

struct Sys {
    int N = 0, n_nuc = 0, n_ao = 0, n_mo = 0;
    std::vector<int> spins, occ, species, init_nuc;
    std::vector<V3> R;
    std::vector<double> Z;
    int basis = 0;
    std::vector<AO> ao;
    std::vector<double> pexp, pcoef;
    std::vector<int> ppow;
    std::vector<double> C;      // effective MO coefficients (rotations applied)
    std::vector<double> C0;     // un-rotated MO coefficients
    int jk = 0;
    double F = 1.0;
    double jas[8] = {0};
    std::vector<int> rot_occ, rot_virt;
    std::vector<double> rot_angle;
    int quirks = 0;
    double init_sigma = 0.5;
    // sector bookkeeping: electrons of each spin in ascending reference order
    std::vector<int> sec[2];    // sec[0] = spin +1, sec[1] = spin -1
    // periodic electron gas (basis kind 2): plane waves e^{i k.r}
    bool pw = false;
    double L = 0.0, rs = 0.0, alphaL = 5.0;
    int kmax = 8, form = 1;
    std::vector<V3> kvec;       // [n_mo] orbital wave vectors

    void apply_rotations() {
        C = C0;
        for (size_t p = 0; p < rot_occ.size(); ++p) {
            int k = rot_occ[p], v = rot_virt[p];
            double c = std::cos(rot_angle[p]), s = std::sin(rot_angle[p]);
            for (int a = 0; a < n_ao; ++a)
                C[(size_t)k * n_ao + a] = c * C0[(size_t)k * n_ao + a] + s * C0[(size_t)v * n_ao + a];
        }
    }
};

Sys make_sys(const orc_system_desc* d) {
    Sys s;
    s.N = d->n_elec;
    s.spins.assign(d->spins, d->spins + s.N);
    s.n_nuc = d->n_nuc;
    for (int I = 0; I < s.n_nuc; ++I) {
        s.R.push_back({d->nuc_pos[3 * I], d->nuc_pos[3 * I + 1], d->nuc_pos[3 * I + 2]});
        s.Z.push_back(d->nuc_charge[I]);
        s.species.push_back(d->nuc_species ? d->nuc_species[I] : 0);
    }
    s.basis = d->basis_kind;
    if (s.basis == 2) {
        // periodic electron gas: mo_coef holds the wave vectors [n_mo][3]
        s.pw = true;
        s.L = d->box_L;
        s.n_mo = d->n_mo;
        for (int k = 0; k < s.n_mo; ++k) s.kvec.push_back({d->mo_coef[3 * k], d->mo_coef[3 * k + 1], d->mo_coef[3 * k + 2]});
        s.occ.assign(d->occ, d->occ + s.N);
        s.jk = d->jastrow_kind;
        s.F = d->jas_F;
        for (int i = 0; i < 8; ++i) s.jas[i] = d->jas[i];
        s.form = (int)d->jas[0];
        s.alphaL = d->jas[4] > 0 ? d->jas[4] : 5.0;
        s.kmax = d->jas[5] > 0 ? (int)d->jas[5] : 8;
        s.quirks = d->quirks;
        s.rs = s.L / std::cbrt(4.0 * M_PI * s.N / 3.0);
        s.init_sigma = d->init_sigma;
        s.init_nuc.assign(s.N, -1);
        for (int e = 0; e < s.N; ++e) s.sec[s.spins[e] > 0 ? 0 : 1].push_back(e);
        return s;
    }
    s.n_ao = d->n_ao;
    for (int a = 0; a < s.n_ao; ++a)
        s.ao.push_back({d->ao_nuc[a], d->ao_l[a], d->ao_m[a], d->ao_prim_off[a], d->ao_prim_off[a + 1]});
    int np = d->ao_prim_off[s.n_ao];
    s.pexp.assign(d->prim_exp, d->prim_exp + np);
    s.pcoef.assign(d->prim_coef, d->prim_coef + np);
    if (d->prim_pow) s.ppow.assign(d->prim_pow, d->prim_pow + np);
    else s.ppow.assign(np, 0);
    s.n_mo = d->n_mo;
    s.C0.assign(d->mo_coef, d->mo_coef + (size_t)s.n_mo * s.n_ao);
    s.occ.assign(d->occ, d->occ + s.N);
    s.jk = d->jastrow_kind;
    s.F = d->jas_F;
    for (int i = 0; i < 8; ++i) s.jas[i] = d->jas[i];
    for (int p = 0; p < d->n_rot; ++p) {
        s.rot_occ.push_back(d->rot_occ[p]);
        s.rot_virt.push_back(d->rot_virt[p]);
        s.rot_angle.push_back(d->rot_angle[p]);
    }
    s.quirks = d->quirks;
    if (d->init_nuc) s.init_nuc.assign(d->init_nuc, d->init_nuc + s.N);
    else s.init_nuc.assign(s.N, -1);
    s.init_sigma = d->init_sigma;
    for (int e = 0; e < s.N; ++e) s.sec[s.spins[e] > 0 ? 0 : 1].push_back(e);
    s.apply_rotations();
    return s;
}

// ---------------------------------------------------------------------------
// Basis functions.
// Contracted Gaussians follow src/systems/methane.rs:498-590 (CGTO::evaluate,
// gradient, laplacian; raw primitive coefficients, no normalisation).
// Slater-type orbitals follow src/wavefunction/slater.rs:91-145 (STO) and
// :17-42 (Slater1s = one primitive with power 0).
// ---------------------------------------------------------------------------
double ao_value(const Sys& s, int a, V3 r) {
    const AO& A = s.ao[a];
    V3 dr = r - s.R[A.nuc];
    if (s.basis == 0) {
        double r2 = dot(dr, dr);
        double ang = A.l == 1 ? comp(dr, A.m) : 1.0;
        double rad = 0.0;
        for (int p = A.p0; p < A.p1; ++p) rad += s.pcoef[p] * std::exp(-s.pexp[p] * r2);
        return ang * rad;
    }
    double d = norm(dr), v = 0.0;
    for (int p = A.p0; p < A.p1; ++p) v += s.pcoef[p] * std::pow(d, s.ppow[p]) * std::exp(-s.pexp[p] * d);
    return v;
}

V3 ao_grad(const Sys& s, int a, V3 r) {
    const AO& A = s.ao[a];
    V3 dr = r - s.R[A.nuc];
    if (s.basis == 0) {
        double r2 = dot(dr, dr), rad = 0.0, rada = 0.0;
        for (int p = A.p0; p < A.p1; ++p) {
            double e = std::exp(-s.pexp[p] * r2);
            rad += s.pcoef[p] * e;
            rada += s.pcoef[p] * s.pexp[p] * e;
        }
        V3 g = (-2.0 * rada) * dr;
        if (A.l == 0) return g;
        V3 out = comp(dr, A.m) * g;
        add_comp(out, A.m, rad);
        return out;
    }
    double d = norm(dr);
    if (d == 0.0) return {0, 0, 0};
    double rd = 0.0;
    for (int p = A.p0; p < A.p1; ++p) {
        double pf = s.ppow[p], z = s.pexp[p];
        double sp = std::pow(d, s.ppow[p]);
        rd += s.pcoef[p] * std::exp(-z * d) * (-z * sp + pf * sp / d);
    }
    return (rd / d) * dr;
}

double ao_lap(const Sys& s, int a, V3 r) {
    const AO& A = s.ao[a];
    V3 dr = r - s.R[A.nuc];
    if (s.basis == 0) {
        double r2 = dot(dr, dr), lr = 0.0, rada = 0.0;
        for (int p = A.p0; p < A.p1; ++p) {
            double al = s.pexp[p], e = std::exp(-al * r2);
            lr += s.pcoef[p] * (-6.0 * al + 4.0 * al * al * r2) * e;
            rada += s.pcoef[p] * al * e;
        }
        if (A.l == 0) return lr;
        double xm = comp(dr, A.m);
        return xm * lr + 2.0 * (-2.0 * xm * rada);
    }
    double d = norm(dr);
    if (d == 0.0) return 0.0;
    double v = 0.0;
    for (int p = A.p0; p < A.p1; ++p) {
        double pf = s.ppow[p], z = s.pexp[p];
        double sp = std::pow(d, s.ppow[p]), sp1 = sp / d, sp2 = sp1 / d;
        double d2 = z * z * sp - 2.0 * z * pf * sp1 + pf * (pf - 1.0) * sp2;
        double d1 = 2.0 * (-z * sp + pf * sp1) / d;
        v += s.pcoef[p] * std::exp(-z * d) * (d2 + d1);
    }
    return v;
}

// MO evaluation, literal: every AO re-evaluated for every MO
// (src/systems/methane.rs:781-809).
double mo_value(const Sys& s, const std::vector<double>& C, int k, V3 r) {
    double v = 0.0;
    for (int a = 0; a < s.n_ao; ++a) v += C[(size_t)k * s.n_ao + a] * ao_value(s, a, r);
    return v;
}
V3 mo_grad(const Sys& s, const std::vector<double>& C, int k, V3 r) {
    V3 g{0, 0, 0};
    for (int a = 0; a < s.n_ao; ++a) g = g + C[(size_t)k * s.n_ao + a] * ao_grad(s, a, r);
    return g;
}
double mo_lap(const Sys& s, const std::vector<double>& C, int k, V3 r) {
    double v = 0.0;
    for (int a = 0; a < s.n_ao; ++a) v += C[(size_t)k * s.n_ao + a] * ao_lap(s, a, r);
    return v;
}

// ---------------------------------------------------------------------------
// Dense LU with partial pivoting (restates nalgebra's determinant/try_inverse,
// which the reference calls at src/systems/methane.rs:828-829).
// ---------------------------------------------------------------------------
bool lu_inverse(std::vector<double> A, int n, std::vector<double>& inv, double& logdet, int& sign) {
    std::vector<int> piv(n);
    sign = 1;
    logdet = 0.0;
    for (int k = 0; k < n; ++k) {
        int p = k;
        double best = std::fabs(A[k * n + k]);
        for (int i = k + 1; i < n; ++i)
            if (std::fabs(A[i * n + k]) > best) { best = std::fabs(A[i * n + k]); p = i; }
        piv[k] = p;
        if (best == 0.0) { logdet = -INFINITY; sign = 0; return false; }
        if (p != k) {
            for (int j = 0; j < n; ++j) std::swap(A[k * n + j], A[p * n + j]);
            sign = -sign;
        }
        double d = A[k * n + k];
        if (d < 0) sign = -sign;
        logdet += std::log(std::fabs(d));
        for (int i = k + 1; i < n; ++i) {
            double f = A[i * n + k] / d;
            A[i * n + k] = f;
            for (int j = k + 1; j < n; ++j) A[i * n + j] -= f * A[k * n + j];
        }
    }
    // inverse: solve A X = I column by column (rows of identity permuted)
    inv.assign((size_t)n * n, 0.0);
    std::vector<double> b(n);
    for (int c = 0; c < n; ++c) {
        for (int i = 0; i < n; ++i) b[i] = (i == c) ? 1.0 : 0.0;
        for (int k = 0; k < n; ++k) if (piv[k] != k) std::swap(b[k], b[piv[k]]);
        for (int i = 0; i < n; ++i) { double v = b[i]; for (int j = 0; j < i; ++j) v -= A[i * n + j] * b[j]; b[i] = v; }
        for (int i = n - 1; i >= 0; --i) { double v = b[i]; for (int j = i + 1; j < n; ++j) v -= A[i * n + j] * b[j]; b[i] = v / A[i * n + i]; }
        for (int i = 0; i < n; ++i) inv[(size_t)i * n + c] = b[i];
    }
    return true;
}

// One spin sector (src/systems/methane.rs:812-831): S[row][col] = phi_col(r_row),
// where col runs over the sector's electrons and phi_col = MO occ[electron].
struct Sector { int n; std::vector<double> inv; double logdet; int sign; bool ok; };
Sector slater_sector(const Sys& s, const std::vector<double>& C, const std::vector<V3>& r, int sp) {
    const std::vector<int>& idx = s.sec[sp];
    int n = (int)idx.size();
    Sector out;
    out.n = n;
    if (n == 0) { out.logdet = 0; out.sign = 1; out.ok = true; return out; }
    std::vector<double> S((size_t)n * n);
    for (int row = 0; row < n; ++row)
        for (int col = 0; col < n; ++col) S[(size_t)row * n + col] = mo_value(s, C, s.occ[idx[col]], r[idx[row]]);
    out.ok = lu_inverse(S, n, out.inv, out.logdet, out.sign);
    return out;
}

// ---------------------------------------------------------------------------
// Jastrow factors, in the log domain (u = ln J).
// PADE_F is Jastrow1 (src/correlation/jastrow.rs:15-54) for two electrons and
// Jastrow2 (:60-126) for more; quirk bits reproduce Jastrow2's gradient
// prefactor (:102) and per-pair Laplacian (:110-125).
// PADE_EEN is Jastrow3 (:138-449) with per-spin-class b and per-species e-n
// coefficients; the reference form is b_anti=b_para=b_ee, A0=A1=1, B0=B1=b_en.
// ---------------------------------------------------------------------------
struct JOut { double u; std::vector<V3> g; std::vector<double> lap; };  // lap = grad^2 J / J

JOut jastrow(const Sys& s, const std::vector<V3>& r) {
    int N = s.N;
    JOut o;
    o.u = 0.0;
    o.g.assign(N, {0, 0, 0});
    o.lap.assign(N, 0.0);
    std::vector<double> lu(N, 0.0), gsq(N, 0.0);
    if (s.jk == 1) {
        double F = s.F;
        double gfac = (s.quirks & 1) ? F : 1.0;
        for (int i = 0; i < N; ++i)
            for (int j = i + 1; j < N; ++j) {
                V3 rij = r[i] - r[j];
                double d = norm(rij), f = 1.0 + d / F;
                o.u += -F / (2.0 * f);
                double up = 1.0 / (2.0 * f * f);          // du/dr
                V3 gi = (gfac * up / d) * rij;
                o.g[i] = o.g[i] + gi;
                o.g[j] = o.g[j] - gi;
                double l = 1.0 / (d * f * f * f);         // u'' + 2u'/r
                lu[i] += l; lu[j] += l;
                gsq[i] += up * up; gsq[j] += up * up;
            }
        for (int i = 0; i < N; ++i)
            o.lap[i] = (s.quirks & 2) ? (gsq[i] + lu[i]) : (dot(o.g[i], o.g[i]) / (gfac * gfac) + lu[i]);
        return o;
    }
    if (s.jk == 2) {
        const double* p = s.jas;   // b_anti b_para a_anti a_para B0 B1 A0 A1
        for (int i = 0; i < N; ++i)
            for (int j = i + 1; j < N; ++j) {
                bool para = s.spins[i] == s.spins[j];
                double a = para ? p[3] : p[2], b = para ? p[1] : p[0];
                V3 rij = r[i] - r[j];
                double d = norm(rij);
                o.u += a * d / (1.0 + b * d);
                if (d < 1e-10) continue;                  // jastrow.rs:256
                double den = 1.0 + b * d;
                V3 gi = (a / (den * den * d)) * rij;
                o.g[i] = o.g[i] + gi;
                o.g[j] = o.g[j] - gi;
                double l = 2.0 * a / (d * den * den) - 2.0 * a * b / (den * den * den);
                lu[i] += l; lu[j] += l;
            }
        for (int i = 0; i < N; ++i)
            for (int I = 0; I < s.n_nuc; ++I) {
                int sp = s.species[I];
                double A = p[6 + sp] * s.Z[I], B = p[4 + sp];
                V3 riI = r[i] - s.R[I];
                double d = norm(riI);
                o.u -= A * d / (1.0 + B * d);
                if (d < 1e-10) continue;                  // jastrow.rs:277
                double den = 1.0 + B * d;
                o.g[i] = o.g[i] + (-A / (den * den * d)) * riI;
                lu[i] += -2.0 * A / (d * den * den) + 2.0 * A * B / (den * den * den);
            }
        for (int i = 0; i < N; ++i) o.lap[i] = lu[i] + dot(o.g[i], o.g[i]);
        return o;
    }
    return o;
}

// ---------------------------------------------------------------------------
// Full evaluation of one configuration.
// ---------------------------------------------------------------------------
struct Eval {
    double logabs; int sign; bool ok;
    std::vector<V3> grad;       // grad_i psi / psi
    std::vector<double> lap;    // lap_i psi / psi
    double el;
    Sector sec[2];
    JOut J;
};

double potential(const Sys& s, const std::vector<V3>& r) {
    double v = 0.0;
    for (int i = 0; i < s.N; ++i)
        for (int I = 0; I < s.n_nuc; ++I) v += -s.Z[I] / norm(r[i] - s.R[I]);
    for (int i = 0; i < s.N; ++i)
        for (int j = i + 1; j < s.N; ++j) v += 1.0 / norm(r[i] - r[j]);
    for (int I = 0; I < s.n_nuc; ++I)
        for (int J = I + 1; J < s.n_nuc; ++J) v += s.Z[I] * s.Z[J] / norm(s.R[I] - s.R[J]);
    return v;
}


// ---------------------------------------------------------------------------
// Homogeneous electron gas (src/systems/heg.rs): complex plane-wave spin
// determinants, spin-dependent Jastrow with a minimum-image cutoff at L/2,
// Ewald Coulomb energy.  Quirk bits: 4 = the reference's Ewald (alpha = 5/L,
// |n_i| <= 7 cube, minimum image only, Madelung -0.448 N / r_s, heg.rs:526-581);
// 8 = the reference's cross term without the orbital factor (heg.rs:711-720).
// Without them: the one-component-plasma Ewald sum with its self and
// background terms, and the exact cross term.
// ---------------------------------------------------------------------------
typedef std::complex<double> cplx;

V3 min_image(const Sys& s, V3 v) {
    return {v.x - s.L * std::round(v.x / s.L), v.y - s.L * std::round(v.y / s.L), v.z - s.L * std::round(v.z / s.L)};
}

// u, du/dr, lap u of the three forms (heg.rs:352-444); a = cusp amplitude
void heg_pair(const Sys& s, double r, double a, double& u, double& du, double& lu) {
    double f = s.F;
    if (s.form == 0) {                      // Pade
        u = a * r / (1.0 + r / f);
        du = a * f * f / ((f + r) * (f + r));
        lu = 2.0 * a * f * f * f / (r * (f + r) * (f + r) * (f + r));
    } else if (s.form == 1) {               // RPA
        double b = 1.0 / f, c = 0.2 / (f * f);
        double den = 1.0 + b * r + c * r * r;
        u = a * r / den;
        du = a * (1.0 - c * r * r) / (den * den);
        double d2 = -a * 2.0 * (c * r * den + (1.0 - c * r * r) * (b + 2.0 * c * r)) / (den * den * den);
        lu = d2 + 2.0 / r * du;
    } else {                                // Yukawa
        double x = r / f, ex = std::exp(-x);
        u = a * r * ex / (1.0 + x);
        du = a * ex * (1.0 - x - x * x) / ((1.0 + x) * (1.0 + x));
        double d2 = a * ex / (f * f * (1.0 + x) * (1.0 + x) * (1.0 + x)) * (-3.0 - 3.0 * x + x * x + x * x * x);
        lu = d2 + 2.0 / r * du;
    }
}

struct HegSector { int n; std::vector<cplx> inv, M; double logabs; bool ok; };

// M[row][col] = e^{i k_col . r_row}; complex Gauss-Jordan with partial pivoting
HegSector heg_sector(const Sys& s, const std::vector<V3>& r, int sp) {
    const std::vector<int>& idx = s.sec[sp];
    int n = (int)idx.size();
    HegSector o;
    o.n = n; o.logabs = 0.0; o.ok = true;
    o.M.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i)
        for (int c = 0; c < n; ++c) {
            V3 k = s.kvec[s.occ[idx[c]]];
            double ph = dot(k, r[idx[i]]);
            o.M[(size_t)i * n + c] = cplx(std::cos(ph), std::sin(ph));
        }
    std::vector<cplx> A = o.M, I((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) I[(size_t)i * n + i] = 1.0;
    for (int k = 0; k < n; ++k) {
        int p = k;
        for (int i = k + 1; i < n; ++i) if (std::abs(A[(size_t)i * n + k]) > std::abs(A[(size_t)p * n + k])) p = i;
        if (p != k) for (int j = 0; j < n; ++j) { std::swap(A[(size_t)k * n + j], A[(size_t)p * n + j]); std::swap(I[(size_t)k * n + j], I[(size_t)p * n + j]); }
        cplx piv = A[(size_t)k * n + k];
        if (std::abs(piv) == 0.0) { o.ok = false; o.logabs = -INFINITY; return o; }
        o.logabs += std::log(std::abs(piv));
        cplx ip = 1.0 / piv;
        for (int j = 0; j < n; ++j) { A[(size_t)k * n + j] *= ip; I[(size_t)k * n + j] *= ip; }
        for (int i = 0; i < n; ++i) {
            if (i == k) continue;
            cplx f = A[(size_t)i * n + k];
            for (int j = 0; j < n; ++j) { A[(size_t)i * n + j] -= f * A[(size_t)k * n + j]; I[(size_t)i * n + j] -= f * I[(size_t)k * n + j]; }
        }
    }
    o.inv = I;                  // inv[k][i]: orbital row k, electron column i
    return o;
}

double heg_jastrow(const Sys& s, const std::vector<V3>& r, std::vector<V3>* g, std::vector<double>* lu) {
    double u = 0.0;
    if (g) g->assign(s.N, {0, 0, 0});
    if (lu) lu->assign(s.N, 0.0);
    for (int i = 0; i < s.N; ++i)
        for (int j = i + 1; j < s.N; ++j) {
            V3 rij = min_image(s, r[i] - r[j]);
            double d = norm(rij);
            if (!(d < s.L / 2.0 && d > 1e-10)) continue;          // heg.rs:468-470
            double a = (s.spins[i] == s.spins[j]) ? s.jas[3] : s.jas[2];
            double uu, du, l;
            heg_pair(s, d, a, uu, du, l);
            u += uu;
            if (g) { V3 gg = (du / d) * rij; (*g)[i] = (*g)[i] + gg; (*g)[j] = (*g)[j] - gg; }
            if (lu) { (*lu)[i] += l; (*lu)[j] += l; }
        }
    return u;
}


// Per-electron constant of the one-component-plasma Ewald energy: half the
// interaction with its own images, the self term and the background term:
// (1/2) sum_{n!=0} erfc(alpha nL)/(nL) - alpha/sqrt(pi) - pi N / (2 V alpha^2).
double heg_madelung_self(const Sys& s) {
    const double L = s.L, alpha = s.alphaL / L, V = L * L * L;
    double img = 0.0;
    for (int a = -3; a <= 3; ++a)
        for (int b = -3; b <= 3; ++b)
            for (int c = -3; c <= 3; ++c) {
                if (!a && !b && !c) continue;
                double d = L * std::sqrt((double)(a * a + b * b + c * c));
                img += std::erfc(alpha * d) / d;
            }
    // the reciprocal i == j terms are inside |rho_k|^2 of heg_ewald
    return 0.5 * img - alpha / std::sqrt(M_PI) - M_PI * s.N / (2.0 * V * alpha * alpha);
}

double heg_ewald(const Sys& s, const std::vector<V3>& r) {
    const int N = s.N;
    const double L = s.L, V = L * L * L;
    if (s.quirks & 4) {                    // heg.rs:526-581
        double alpha = 5.0 / L, vr = 0.0, vk = 0.0;
        for (int i = 0; i < N; ++i)
            for (int j = i + 1; j < N; ++j) {
                double d = norm(min_image(s, r[i] - r[j]));
                if (d > 1e-10) vr += std::erfc(alpha * d) / d;
            }
        double dk = 2.0 * M_PI / L;
        for (int nx = -7; nx <= 7; ++nx)
            for (int ny = -7; ny <= 7; ++ny)
                for (int nz = -7; nz <= 7; ++nz) {
                    if (!nx && !ny && !nz) continue;
                    V3 k{nx * dk, ny * dk, nz * dk};
                    double k2 = dot(k, k);
                    double fac = 4.0 * M_PI / (V * k2) * std::exp(-k2 / (4.0 * alpha * alpha));
                    cplx rho = 0.0;
                    for (int i = 0; i < N; ++i) { double ph = dot(k, r[i]); rho += cplx(std::cos(ph), std::sin(ph)); }
                    vk += 0.5 * fac * (std::norm(rho) - N);
                }
        return vr + vk - N * 0.448 / s.rs;
    }
    // one-component plasma: electrons in a uniform neutralising background
    const double alpha = s.alphaL / L;
    const double rcut = 5.6 / alpha;       // erfc(5.6) < 1e-14
    double vr = 0.0;
    for (int i = 0; i < N; ++i)
        for (int j = i + 1; j < N; ++j) {
            V3 d0 = min_image(s, r[i] - r[j]);
            for (int a = -1; a <= 1; ++a)
                for (int b = -1; b <= 1; ++b)
                    for (int c = -1; c <= 1; ++c) {
                        V3 d{d0.x + a * L, d0.y + b * L, d0.z + c * L};
                        double dn = norm(d);
                        if (dn < rcut) vr += std::erfc(alpha * dn) / dn;
                    }
        }
    double vk = 0.0, dk = 2.0 * M_PI / L;
    const int K = s.kmax;
    for (int nx = 0; nx <= K; ++nx)
        for (int ny = -K; ny <= K; ++ny)
            for (int nz = -K; nz <= K; ++nz) {
                // half space: nx > 0, or nx == 0 and (ny > 0 or ny == 0 and nz > 0)
                if (nx == 0 && (ny < 0 || (ny == 0 && nz <= 0))) continue;
                if (nx * nx + ny * ny + nz * nz > K * K) continue;
                V3 k{nx * dk, ny * dk, nz * dk};
                double k2 = dot(k, k);
                cplx rho = 0.0;
                for (int i = 0; i < N; ++i) { double ph = dot(k, r[i]); rho += cplx(std::cos(ph), std::sin(ph)); }
                vk += 2.0 * (2.0 * M_PI / V) * std::exp(-k2 / (4.0 * alpha * alpha)) / k2 * std::norm(rho);
            }
    return vr + vk + N * heg_madelung_self(s);
}

struct HegEval { double logabs; bool ok; std::vector<V3> grad; std::vector<double> lap; double el; };

// evaluate / local_energy of heg.rs:867-934 in the log domain; grad is
// Re(grad_i psi / psi) (heg.rs:887-889 takes it numerically from |psi|),
// lap is Re(lap_i psi / psi), el = -1/2 sum lap + V.
HegEval heg_evaluate(const Sys& s, const std::vector<V3>& r) {
    HegEval o;
    o.grad.assign(s.N, {0, 0, 0});
    o.lap.assign(s.N, 0.0);
    std::vector<V3> gu;
    std::vector<double> lu;
    double u = heg_jastrow(s, r, &gu, &lu);
    o.logabs = u;
    o.ok = true;
    double kin = 0.0;
    for (int sp = 0; sp < 2; ++sp) {
        HegSector sec = heg_sector(s, r, sp);
        o.ok = o.ok && sec.ok;
        o.logabs += sec.logabs;
        const std::vector<int>& idx = s.sec[sp];
        int n = sec.n;
        for (int i = 0; i < n; ++i) {
            int e = idx[i];
            cplx gx = 0.0, gy = 0.0, gz = 0.0, l = 0.0, qx = 0.0, qy = 0.0, qz = 0.0;
            for (int c = 0; c < n; ++c) {
                V3 k = s.kvec[s.occ[idx[c]]];
                cplx w = sec.inv[(size_t)c * n + i];
                cplx wf = w * sec.M[(size_t)i * n + c];
                cplx ik(0.0, 1.0);
                gx += wf * ik * k.x; gy += wf * ik * k.y; gz += wf * ik * k.z;
                l += wf * (-dot(k, k));
                qx += w * ik * k.x; qy += w * ik * k.y; qz += w * ik * k.z;      // reference: no orbital factor
            }
            V3 gd{gx.real(), gy.real(), gz.real()};
            V3 gc = (s.quirks & 8) ? V3{qx.real(), qy.real(), qz.real()} : gd;
            o.grad[e] = gd + gu[e];
            o.lap[e] = l.real() + lu[e] + dot(gu[e], gu[e]) + 2.0 * dot(gc, gu[e]);
            kin += o.lap[e];
        }
    }
    o.el = -0.5 * kin + heg_ewald(s, r);
    return o;
}
// log|psi| only (the reference's evaluate(), src/systems/methane.rs:1122-1124).
double log_psi(const Sys& s, const std::vector<V3>& r, int& sign, bool& ok) {
    if (s.pw) {
        double la = heg_jastrow(s, r, nullptr, nullptr);
        ok = true;
        for (int sp = 0; sp < 2; ++sp) { HegSector sec = heg_sector(s, r, sp); la += sec.logabs; ok = ok && sec.ok; }
        sign = 1;
        return la;
    }
    Sector a = slater_sector(s, s.C, r, 0), b = slater_sector(s, s.C, r, 1);
    JOut J = jastrow(s, r);
    sign = a.sign * b.sign;
    ok = a.ok && b.ok;
    return a.logdet + b.logdet + J.u;
}

// derivative(), laplacian(), local_energy(): src/systems/methane.rs:1126-1181,
// src/systems/lithium.rs:30-81, src/systems/hydrogen.rs:126-200.
Eval evaluate_full(const Sys& s, const std::vector<V3>& r) {
    Eval e;
    if (s.pw) {
        HegEval h = heg_evaluate(s, r);
        e.logabs = h.logabs; e.sign = 1; e.ok = h.ok; e.grad = h.grad; e.lap = h.lap; e.el = h.el;
        return e;
    }
    e.sec[0] = slater_sector(s, s.C, r, 0);
    e.sec[1] = slater_sector(s, s.C, r, 1);
    e.J = jastrow(s, r);
    e.ok = e.sec[0].ok && e.sec[1].ok;
    e.sign = e.sec[0].sign * e.sec[1].sign;
    e.logabs = e.sec[0].logdet + e.sec[1].logdet + e.J.u;
    e.grad.assign(s.N, {0, 0, 0});
    e.lap.assign(s.N, 0.0);
    double kin = 0.0;
    for (int sp = 0; sp < 2; ++sp) {
        const std::vector<int>& idx = s.sec[sp];
        int n = (int)idx.size();
        for (int row = 0; row < n; ++row) {
            int el = idx[row];
            V3 gd{0, 0, 0};
            double ld = 0.0;
            for (int col = 0; col < n; ++col) {
                double w = e.sec[sp].inv[(size_t)col * n + row];
                int k = s.occ[idx[col]];
                gd = gd + w * mo_grad(s, s.C, k, r[el]);
                ld += w * mo_lap(s, s.C, k, r[el]);
            }
            V3 gj = e.J.g[el];
            e.grad[el] = gd + gj;
            e.lap[el] = ld + 2.0 * dot(gd, gj) + e.J.lap[el];
            kin += e.lap[el];
        }
    }
    e.el = -0.5 * kin + potential(s, r);
    return e;
}

// Parameter log-derivatives O_p = d ln|psi| / dp, generalising
// Jastrow3::d_ln_j_d_* (src/correlation/jastrow.rs:326-391) to the
// per-class / per-species parameters, plus MO-rotation angles.
void log_derivs(const Sys& s, const std::vector<V3>& r, double* O) {
    for (int p = 0; p < 8; ++p) O[p] = 0.0;
    if (s.jk == 2) {
        const double* p = s.jas;
        for (int i = 0; i < s.N; ++i)
            for (int j = i + 1; j < s.N; ++j) {
                bool para = s.spins[i] == s.spins[j];
                double a = para ? p[3] : p[2], b = para ? p[1] : p[0];
                double d = norm(r[i] - r[j]), den = 1.0 + b * d;
                O[para ? 1 : 0] += -a * d * d / (den * den);
                O[para ? 3 : 2] += d / den;
            }
        for (int i = 0; i < s.N; ++i)
            for (int I = 0; I < s.n_nuc; ++I) {
                int sp = s.species[I];
                double A = p[6 + sp], B = p[4 + sp], Zi = s.Z[I];
                double d = norm(r[i] - s.R[I]), den = 1.0 + B * d;
                O[4 + sp] += A * Zi * d * d / (den * den);
                O[6 + sp] += -Zi * d / den;
            }
    }
    int nrot = (int)s.rot_occ.size();
    if (!nrot) return;
    // d phi_k / d theta = -sin(t) C0_k + cos(t) C0_v
    std::vector<double> dC((size_t)s.n_mo * s.n_ao, 0.0);
    for (int q = 0; q < nrot; ++q) {
        int k = s.rot_occ[q], v = s.rot_virt[q];
        double c = std::cos(s.rot_angle[q]), sn = std::sin(s.rot_angle[q]);
        for (int a = 0; a < s.n_ao; ++a)
            dC[(size_t)k * s.n_ao + a] = -sn * s.C0[(size_t)k * s.n_ao + a] + c * s.C0[(size_t)v * s.n_ao + a];
    }
    Sector sc[2] = {slater_sector(s, s.C, r, 0), slater_sector(s, s.C, r, 1)};
    for (int q = 0; q < nrot; ++q) {
        int k = s.rot_occ[q];
        double acc = 0.0;
        for (int sp = 0; sp < 2; ++sp) {
            const std::vector<int>& idx = s.sec[sp];
            int n = (int)idx.size();
            for (int col = 0; col < n; ++col) {
                if (s.occ[idx[col]] != k) continue;
                for (int row = 0; row < n; ++row)
                    acc += sc[sp].inv[(size_t)col * n + row] * mo_value(s, dC, k, r[idx[row]]);
            }
        }
        O[8 + q] = acc;
    }
}

// Parameter derivatives of the local energy, dE_L / dp, in the order of
// log_derivs.  The reference has no such function; its SR sampling
// (src/sampling/sr_optimize.rs:104-246) and EnergyCalculator::local_energy
// (src/systems/methane.rs:1154-1182) define what is differentiated:
//   E_L = -1/2 sum_i lap_i psi / psi + V,  lap_i psi / psi = l_i + 2 g_i . j_i + lu_i + |j_i|^2
// with g_i, l_i the determinant's gradient and Laplacian (over psi_D) and j_i,
// lu_i the Jastrow's.  V does not depend on p, so
//   Jastrow p:  dE_L/dp = -1/2 sum_i [ d lu_i/dp + 2 (g_i + j_i) . d j_i/dp ]
//   rotation q (column c of a sector, d phi_c/d theta = psi_c):
//     with B = A^-1, beta = B psi_c(r_.), for X in {grad, lap} of the MOs,
//     d (X B)_ii = X_psi(r_i) B_ci - B_ci sum_k X_k(r_i) beta_k,
//     dE_L/dq = -1/2 sum_i [ d (L B)_ii + 2 d (G B)_ii . j_i ].
// Checked in the tests against central finite differences of E_L.
void el_derivs(const Sys& s, const std::vector<V3>& r, double* dE) {
    int nrot = (int)s.rot_occ.size();
    for (int p = 0; p < 8 + nrot; ++p) dE[p] = 0.0;
    Eval ev = evaluate_full(s, r);
    if (s.jk == 2) {
        const double* p = s.jas;
        for (int i = 0; i < s.N; ++i)
            for (int j = i + 1; j < s.N; ++j) {
                bool para = s.spins[i] == s.spins[j];
                int c = para ? 1 : 0;
                double a = p[2 + c], b = p[c];
                V3 rij = r[i] - r[j];
                double d = norm(rij);
                if (d < 1e-10) continue;
                double den = 1.0 + b * d;
                double gdot = dot(ev.grad[i] - ev.grad[j], rij);
                // d/da: j_i gains rij / (den^2 d); lu_i, lu_j gain 2/(d den^2) - 2b/den^3 each
                double fa = 1.0 / (den * den * d), la = 2.0 / (d * den * den) - 2.0 * b / (den * den * den);
                // d/db: j_i gains -2a rij / den^3; lu gains -6a/den^4 each
                double fb = -2.0 * a / (den * den * den), lb = -6.0 * a / (den * den * den * den);
                dE[2 + c] += -0.5 * (2.0 * la + 2.0 * fa * gdot);
                dE[c] += -0.5 * (2.0 * lb + 2.0 * fb * gdot);
            }
        for (int i = 0; i < s.N; ++i)
            for (int I = 0; I < s.n_nuc; ++I) {
                int sp = s.species[I];
                double Zi = s.Z[I], A = p[6 + sp] * Zi, B = p[4 + sp];
                V3 riI = r[i] - s.R[I];
                double d = norm(riI);
                if (d < 1e-10) continue;
                double den = 1.0 + B * d;
                double gdot = dot(ev.grad[i], riI);
                // j_i gains -A riI/(den^2 d); lu_i gains -2A/(d den^2) + 2AB/den^3
                double fA = -Zi / (den * den * d), lA = -2.0 * Zi / (d * den * den) + 2.0 * Zi * B / (den * den * den);
                double fB = 2.0 * A / (den * den * den), lB = 6.0 * A / (den * den * den * den);
                dE[6 + sp] += -0.5 * (lA + 2.0 * fA * gdot);
                dE[4 + sp] += -0.5 * (lB + 2.0 * fB * gdot);
            }
    }
    if (!nrot) return;
    std::vector<double> dC((size_t)s.n_mo * s.n_ao, 0.0);
    for (int q = 0; q < nrot; ++q) {
        int k = s.rot_occ[q], v = s.rot_virt[q];
        double c = std::cos(s.rot_angle[q]), sn = std::sin(s.rot_angle[q]);
        for (int a = 0; a < s.n_ao; ++a)
            dC[(size_t)k * s.n_ao + a] = -sn * s.C0[(size_t)k * s.n_ao + a] + c * s.C0[(size_t)v * s.n_ao + a];
    }
    for (int q = 0; q < nrot; ++q) {
        int k = s.rot_occ[q];
        double acc = 0.0;
        for (int sp = 0; sp < 2; ++sp) {
            const std::vector<int>& idx = s.sec[sp];
            int n = (int)idx.size();
            int c = -1;
            for (int col = 0; col < n; ++col) if (s.occ[idx[col]] == k) c = col;
            if (c < 0) continue;
            const std::vector<double>& B = ev.sec[sp].inv;   // B[col * n + row]
            std::vector<double> beta(n, 0.0);
            for (int col = 0; col < n; ++col)
                for (int row = 0; row < n; ++row) beta[col] += B[(size_t)col * n + row] * mo_value(s, dC, k, r[idx[row]]);
            for (int row = 0; row < n; ++row) {
                V3 ri = r[idx[row]];
                double bci = B[(size_t)c * n + row];
                V3 tg{0, 0, 0};
                double tl = 0.0;
                for (int col = 0; col < n; ++col) {
                    int kc = s.occ[idx[col]];
                    tg = tg + beta[col] * mo_grad(s, s.C, kc, ri);
                    tl += beta[col] * mo_lap(s, s.C, kc, ri);
                }
                V3 dg = bci * mo_grad(s, dC, k, ri) - bci * tg;
                double dl = bci * mo_lap(s, dC, k, ri) - bci * tl;
                acc += dl + 2.0 * dot(dg, ev.J.g[idx[row]]);
            }
        }
        dE[8 + q] = -0.5 * acc;
    }
}

// Hellmann-Feynman force (src/systems/methane.rs:1241-1272).
void hf_force(const Sys& s, const std::vector<V3>& r, double* F) {
    for (int I = 0; I < s.n_nuc; ++I) {
        V3 f{0, 0, 0};
        for (int i = 0; i < s.N; ++i) {
            V3 dr = r[i] - s.R[I];
            double d = norm(dr);
            if (d > 1e-10) f = f + (s.Z[I] / (d * d * d)) * dr;
        }
        for (int J = 0; J < s.n_nuc; ++J) {
            if (J == I) continue;
            V3 dr = s.R[I] - s.R[J];
            double d = norm(dr);
            if (d > 1e-10) f = f - (s.Z[I] * s.Z[J] / (d * d * d)) * dr;
        }
        F[3 * I] = f.x; F[3 * I + 1] = f.y; F[3 * I + 2] = f.z;
    }
}

// Analytic d ln|psi| / dR_I (src/systems/methane.rs:1007-1101): AOs on I move
// with I (d chi / dR_I = -grad_r chi), plus the e-n Jastrow term.
void nuclear_grad(const Sys& s, const std::vector<V3>& r, double* G) {
    Sector sc[2] = {slater_sector(s, s.C, r, 0), slater_sector(s, s.C, r, 1)};
    for (int I = 0; I < s.n_nuc; ++I) {
        V3 g{0, 0, 0};
        for (int sp = 0; sp < 2; ++sp) {
            const std::vector<int>& idx = s.sec[sp];
            int n = (int)idx.size();
            for (int row = 0; row < n; ++row)
                for (int col = 0; col < n; ++col) {
                    int k = s.occ[idx[col]];
                    V3 dphi{0, 0, 0};
                    for (int a = 0; a < s.n_ao; ++a)
                        if (s.ao[a].nuc == I) dphi = dphi - s.C[(size_t)k * s.n_ao + a] * ao_grad(s, a, r[idx[row]]);
                    g = g + sc[sp].inv[(size_t)col * n + row] * dphi;
                }
        }
        if (s.jk == 2) {
            int sp = s.species[I];
            double A = s.jas[6 + sp] * s.Z[I], B = s.jas[4 + sp];
            for (int i = 0; i < s.N; ++i) {
                V3 dr = r[i] - s.R[I];
                double d = norm(dr);
                if (d < 1e-10) continue;
                double den = 1.0 + B * d;
                g = g + (A / (d * den * den)) * dr;
            }
        }
        G[3 * I] = g.x; G[3 * I + 1] = g.y; G[3 * I + 2] = g.z;
    }
}

std::vector<V3> load_cfg(const double* pos, int N) {
    std::vector<V3> r(N);
    for (int i = 0; i < N; ++i) r[i] = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
    return r;
}

template <class Fn>
void parallel_for(int W, int threads, Fn fn) {
    if (threads <= 1 || W < 2) { for (int w = 0; w < W; ++w) fn(w); return; }
    std::vector<std::thread> pool;
    int T = std::min(threads, W);
    for (int t = 0; t < T; ++t)
        pool.emplace_back([&, t]() { for (int w = t; w < W; w += T) fn(w); });
    for (auto& th : pool) th.join();
}

// Internal electron visiting order: spin-up sector first, then spin-down,
// each in ascending reference index (the CUDA kernels use the same order).
std::vector<int> visit_order(const Sys& s) {
    std::vector<int> o = s.sec[0];
    o.insert(o.end(), s.sec[1].begin(), s.sec[1].end());
    return o;
}

V3 limit_drift(V3 F, double tau, double max_drift) {   // src/sampling/vmc.rs:303-311
    V3 d = tau * F;
    double m = norm(d);
    return m > max_drift ? (max_drift / m) * d : d;
}

// One sweep of single-electron moves for one walker (move_kind 2 Gaussian,
// 3 drift-diffusion), with the shared single-draw Philox layout.  With
// fixed_node a proposal that changes the sign of psi is refused (the
// reference's IS-DMC, src/sampling/is_dmc.rs:254, accepts it).
// margin (may be null) receives the smallest relative distance |u - p| / u
// between an acceptance uniform and its acceptance probability: how close the
// walker came to the opposite decision.
int sweep_walker(const Sys& s, const std::vector<int>& order, std::vector<V3>& r, double& lp, int& sg, uint32_t wid,
                 uint64_t st, int move_kind, double step, double tau, double max_drift, uint64_t seed, int fixed_node,
                 double* margin = nullptr) {
    int acc = 0;
    int N = s.N;
    for (int q = 0; q < N; ++q) {
        int e = order[q];
        U4 x = draw(seed, wid, st, (uint32_t)q, TAG_PROPOSE);
        double n0, n1, n2, n3;
        {
            double rr = std::sqrt(-2.0 * std::log(u24(x.v[0] & 0xFFFFFFu)));
            double t = 6.283185307179586476925286766559 * u24(x.v[1] & 0xFFFFFFu);
            n0 = rr * std::cos(t); n1 = rr * std::sin(t);
            rr = std::sqrt(-2.0 * std::log(u24(x.v[2] & 0xFFFFFFu)));
            t = 6.283185307179586476925286766559 * u24(x.v[3] & 0xFFFFFFu);
            n2 = rr * std::cos(t); n3 = rr * std::sin(t);
        }
        double uacc = u24((x.v[0] >> 24) | ((x.v[1] >> 24) << 8) | ((x.v[2] >> 24) << 16));
        V3 eta{n0, n1, n2};
        std::vector<V3> rn = r;
        double logG = 0.0;
        if (move_kind == 2) {
            rn[e] = r[e] + step * eta;
        } else {
            Eval cur = evaluate_full(s, r);
            V3 dl = limit_drift(2.0 * cur.grad[e], tau, max_drift);
            rn[e] = r[e] + dl + std::sqrt(2.0 * tau) * eta;
            Eval nw = evaluate_full(s, rn);
            if (!nw.ok) continue;
            V3 dn = limit_drift(2.0 * nw.grad[e], tau, max_drift);
            V3 fd = rn[e] - r[e] - dl, bd = r[e] - rn[e] - dn;
            logG = (-dot(bd, bd) + dot(fd, fd)) / (4.0 * tau);
        }
        int sgn;
        bool okn;
        double lpn = log_psi(s, rn, sgn, okn);
        if (!okn) continue;
        if (fixed_node && sgn != sg) continue;
        double prob = std::exp(2.0 * (lpn - lp) + logG);
        if (margin) *margin = std::min(*margin, std::fabs(uacc - prob) / uacc);
        if (uacc < prob) {
            if (s.pw) rn[e] = {rn[e].x - s.L * std::floor(rn[e].x / s.L), rn[e].y - s.L * std::floor(rn[e].y / s.L),
                               rn[e].z - s.L * std::floor(rn[e].z / s.L)};
            r = rn; lp = lpn; sg = sgn; ++acc;
        }
    }
    return acc;
}

}  // namespace

extern "C" {

int orc_desc_size(void) { return (int)sizeof(orc_system_desc); }

void orc_philox(const uint32_t* ctr, const uint32_t* key, uint32_t* out) {
    U4 c{{ctr[0], ctr[1], ctr[2], ctr[3]}};
    U4 r = philox(c, key[0], key[1]);
    for (int i = 0; i < 4; ++i) out[i] = r.v[i];
}

// Batched full evaluation: outputs may be NULL.  pos is W x n_elec x 3 in the
// reference electron order.
int orc_eval(const orc_system_desc* d, int W, const double* pos, double* logabs, int* sign,
             double* grad, double* lap, double* el, int threads) {
    Sys s = make_sys(d);
    int N = s.N;
    parallel_for(W, threads, [&](int w) {
        std::vector<V3> r = load_cfg(pos + (size_t)w * N * 3, N);
        Eval e = evaluate_full(s, r);
        if (logabs) logabs[w] = e.logabs;
        if (sign) sign[w] = e.sign;
        for (int i = 0; i < N; ++i) {
            if (grad) { grad[((size_t)w * N + i) * 3] = e.grad[i].x; grad[((size_t)w * N + i) * 3 + 1] = e.grad[i].y; grad[((size_t)w * N + i) * 3 + 2] = e.grad[i].z; }
            if (lap) lap[(size_t)w * N + i] = e.lap[i];
        }
        if (el) el[w] = e.el;
    });
    return 0;
}

// Jastrow alone (value J, gradient grad J, Laplacian lap J) in the reference's
// non-log convention, for the golden checks of src/lib.rs:31-85.
int orc_jastrow(const orc_system_desc* d, const double* pos, double* J, double* gradJ, double* lapJ) {
    Sys s = make_sys(d);
    std::vector<V3> r = load_cfg(pos, s.N);
    JOut o = jastrow(s, r);
    double j = std::exp(o.u);
    *J = j;
    for (int i = 0; i < s.N; ++i) {
        gradJ[3 * i] = j * o.g[i].x; gradJ[3 * i + 1] = j * o.g[i].y; gradJ[3 * i + 2] = j * o.g[i].z;
        lapJ[i] = j * o.lap[i];
    }
    return 0;
}

int orc_logderiv(const orc_system_desc* d, int W, const double* pos, double* O, int threads) {
    Sys s = make_sys(d);
    int P = 8 + (int)s.rot_occ.size();
    parallel_for(W, threads, [&](int w) {
        std::vector<V3> r = load_cfg(pos + (size_t)w * s.N * 3, s.N);
        log_derivs(s, r, O + (size_t)w * P);
    });
    return 0;
}

// dE_L / dp per configuration, [W][8 + n_rot] (el_derivs).
int orc_el_derivs(const orc_system_desc* d, int W, const double* pos, double* dE, int threads) {
    Sys s = make_sys(d);
    int P = 8 + (int)s.rot_occ.size();
    parallel_for(W, threads, [&](int w) {
        std::vector<V3> r = load_cfg(pos + (size_t)w * s.N * 3, s.N);
        el_derivs(s, r, dE + (size_t)w * P);
    });
    return 0;
}

int orc_forces(const orc_system_desc* d, int W, const double* pos, double* F_hf, double* omega, int threads) {
    Sys s = make_sys(d);
    parallel_for(W, threads, [&](int w) {
        std::vector<V3> r = load_cfg(pos + (size_t)w * s.N * 3, s.N);
        if (F_hf) hf_force(s, r, F_hf + (size_t)w * s.n_nuc * 3);
        if (omega) nuclear_grad(s, r, omega + (size_t)w * s.n_nuc * 3);
    });
    return 0;
}

// Finite-difference d ln|psi| / dR_I (src/systems/hydrogen.rs:260-290).
int orc_forces_fd(const orc_system_desc* d, int W, const double* pos, double h, double* omega) {
    Sys s0 = make_sys(d);
    for (int w = 0; w < W; ++w) {
        std::vector<V3> r = load_cfg(pos + (size_t)w * s0.N * 3, s0.N);
        for (int I = 0; I < s0.n_nuc; ++I)
            for (int ax = 0; ax < 3; ++ax) {
                Sys sp = s0, sm = s0;
                add_comp(sp.R[I], ax, h);
                add_comp(sm.R[I], ax, -h);
                int sg; bool ok;
                double lp = log_psi(sp, r, sg, ok), lm = log_psi(sm, r, sg, ok);
                omega[((size_t)w * s0.n_nuc + I) * 3 + ax] = (lp - lm) / (2.0 * h);
            }
    }
    return 0;
}

// Walker initialisation with the shared Philox stream: electron e of walker w
// is placed at N(R_init(e), sigma) (src/systems/methane.rs:1105-1120).
int orc_init(const orc_system_desc* d, int W, uint32_t walker0, uint64_t seed, double* pos) {
    Sys s = make_sys(d);
    for (int w = 0; w < W; ++w)
        for (int e = 0; e < s.N; ++e) {
            U4 x = draw(seed, walker0 + (uint32_t)w, 0, (uint32_t)e, TAG_INIT);
            double n0, n1, n2, n3;
            box_muller(x.v[0], x.v[1], n0, n1);
            box_muller(x.v[2], x.v[3], n2, n3);
            double* p = pos + ((size_t)w * s.N + e) * 3;
            if (s.pw) {   // uniform in the box (heg.rs:841-852)
                p[0] = s.L * u01(x.v[0]); p[1] = s.L * u01(x.v[1]); p[2] = s.L * u01(x.v[2]);
                continue;
            }
            V3 c = s.init_nuc[e] >= 0 ? s.R[s.init_nuc[e]] : V3{0, 0, 0};
            p[0] = c.x + s.init_sigma * n0;
            p[1] = c.y + s.init_sigma * n1;
            p[2] = c.z + s.init_sigma * n2;
        }
    return 0;
}

// Metropolis / drift-diffusion sweeps, reference algorithm with full
// re-evaluation per proposal (src/sampling/vmc.rs:95-119, 339-394).
// move_kind: 0 all-electron Gaussian, 1 all-electron uniform box,
//            2 single-electron Gaussian, 3 single-electron drift-diffusion.
// For all-electron moves one "sweep" is one step; step index = sweep0 + t.
// pos is W x N x 3 in reference order; accepted[w] counts accepted proposals.
// e_local (optional) receives E_L of the final configuration.
// margin (may be NULL) receives per walker the smallest relative distance
// between an acceptance uniform and its acceptance probability over the run.
int orc_sweeps(const orc_system_desc* d, int W, uint32_t walker0, double* pos, int n_sweeps,
               uint64_t sweep0, int move_kind, double step, double tau, double max_drift,
               uint64_t seed, int* accepted, double* e_local, double* margin, int threads) {
    Sys s = make_sys(d);
    int N = s.N;
    std::vector<int> order = visit_order(s);
    parallel_for(W, threads, [&](int w) {
        uint32_t wid = walker0 + (uint32_t)w;
        std::vector<V3> r = load_cfg(pos + (size_t)w * N * 3, N);
        int sg; bool ok;
        double lp = log_psi(s, r, sg, ok);
        int acc = 0;
        double mg = INFINITY;
        for (int t = 0; t < n_sweeps; ++t) {
            uint64_t st = sweep0 + (uint64_t)t;
            if (move_kind == 0 || move_kind == 1) {
                std::vector<V3> rn = r;
                for (int q = 0; q < N; ++q) {
                    int e = order[q];
                    U4 x = draw(seed, wid, st, (uint32_t)q, TAG_PROPOSE);
                    if (move_kind == 0) {
                        double n0, n1, n2, n3;
                        box_muller(x.v[0], x.v[1], n0, n1);
                        box_muller(x.v[2], x.v[3], n2, n3);
                        rn[e] = r[e] + step * V3{n0, n1, n2};
                    } else {
                        rn[e] = r[e] + step * V3{u01(x.v[0]) - 0.5, u01(x.v[1]) - 0.5, u01(x.v[2]) - 0.5};
                    }
                }
                int sgn; bool okn;
                double lpn = log_psi(s, rn, sgn, okn);
                double prob = std::exp(2.0 * (lpn - lp));
                U4 a = draw(seed, wid, st, 0, TAG_ACCEPT);
                if (okn) mg = std::min(mg, std::fabs(u01(a.v[0]) - prob) / u01(a.v[0]));
                if (okn && u01(a.v[0]) < prob) { r = rn; lp = lpn; sg = sgn; ++acc; }
                continue;
            }
            acc += sweep_walker(s, order, r, lp, sg, wid, st, move_kind, step, tau, max_drift, seed, 0, &mg);
        }
        if (margin) margin[w] = mg;
        for (int i = 0; i < N; ++i) {
            double* p = pos + ((size_t)w * N + i) * 3;
            p[0] = r[i].x; p[1] = r[i].y; p[2] = r[i].z;
        }
        if (accepted) accepted[w] = acc;
        if (e_local) e_local[w] = evaluate_full(s, r).el;
    });
    return 0;
}

// Importance-sampled DMC (src/sampling/is_dmc.rs:208-302, 385-502) with the
// shared Philox layout: per step one drift-diffusion sweep per walker made
// with the reference's move at tau_move (variance 2 tau_move; tau_move = tau is
// the reference, tau / 2 the Hartree-unit projector)
// (walker id = its slot in the current population, step index = DMC step),
// E_L after the sweep, copies m = min(floor(exp(tau (E_ref - (E_L + E_old)/2)) + xi), 3)
// with xi from tag-4 draws, populations rebuilt in slot order, and
// E_ref = <E_L> - kappa ln(N / N_target) / tau.  Stops early if the population
// collapses or exceeds `cap`.  Returns the number of steps done; pos_out
// receives the final population, pops/energies the per-step values.  e_cut > 0
// clamps the branching energy (E_L + E_old)/2 to e_ref +- e_cut (an option of
// the device path; the reference branches unclamped).
int orc_dmc(const orc_system_desc* d, int W0, const double* pos_in, int n_steps, uint64_t step0, double tau,
            double tau_move, double max_drift, int fixed_node, double kappa, double e_cut, int target, uint64_t seed,
            int cap, double* pos_out,
            int* W_out, int* pops, double* energies, double* e_ref_io, int threads) {
    Sys s = make_sys(d);
    int N = s.N;
    std::vector<int> order = visit_order(s);
    std::vector<std::vector<V3>> R(W0);
    std::vector<double> E(W0), lpv(W0);
    std::vector<int> sgv(W0);
    for (int w = 0; w < W0; ++w) R[w] = load_cfg(pos_in + (size_t)w * N * 3, N);
    parallel_for(W0, threads, [&](int w) {
        Eval e = evaluate_full(s, R[w]);
        E[w] = e.el; lpv[w] = e.logabs; sgv[w] = e.sign;
    });
    double e_ref = *e_ref_io;
    int t = 0;
    for (; t < n_steps; ++t) {
        uint64_t st = step0 + (uint64_t)t;
        int W = (int)R.size();
        std::vector<double> Eold = E;
        parallel_for(W, threads, [&](int w) {
            sweep_walker(s, order, R[w], lpv[w], sgv[w], (uint32_t)w, st, 3, 0.0, tau_move, max_drift, seed,
                         fixed_node);
            Eval e = evaluate_full(s, R[w]);
            E[w] = e.el; lpv[w] = e.logabs; sgv[w] = e.sign;
        });
        std::vector<std::vector<V3>> R2;
        std::vector<double> E2, lp2;
        std::vector<int> sg2;
        double esum = 0.0;
        for (int w = 0; w < W; ++w) {
            int m = 0;
            if (std::isfinite(E[w]) && std::isfinite(Eold[w])) {
                double eb = 0.5 * (E[w] + Eold[w]);
                if (e_cut > 0.0) eb = std::min(e_ref + e_cut, std::max(e_ref - e_cut, eb));
                double wgt = std::exp(tau * (e_ref - eb));
                U4 x = draw(seed, (uint32_t)w, st, 0, TAG_BRANCH);
                double f = std::floor(wgt + u01(x.v[0]));
                m = f >= 3.0 ? 3 : (int)f;
                if (m < 0) m = 0;
            }
            for (int c = 0; c < m; ++c) {
                R2.push_back(R[w]); E2.push_back(E[w]); lp2.push_back(lpv[w]); sg2.push_back(sgv[w]);
                esum += E[w];
            }
        }
        int Wn = (int)R2.size();
        pops[t] = Wn;
        if (Wn == 0 || Wn > cap) { energies[t] = 0.0; ++t; R.swap(R2); break; }
        double em = esum / Wn;
        energies[t] = em;
        e_ref = em - kappa * std::log((double)Wn / (double)target) / tau;
        R.swap(R2); E.swap(E2); lpv.swap(lp2); sgv.swap(sg2);
    }
    *W_out = (int)R.size();
    for (size_t w = 0; w < R.size() && (int)w < cap; ++w)
        for (int i = 0; i < N; ++i) {
            double* p = pos_out + (w * N + i) * 3;
            p[0] = R[w][i].x; p[1] = R[w][i].y; p[2] = R[w][i].z;
        }
    *e_ref_io = e_ref;
    return t;
}

// HEG Ewald energy of one configuration and the per-electron constant
// (alpha-invariance and Madelung checks).
double orc_heg_ewald(const orc_system_desc* d, const double* pos, double alphaL, int kmax) {
    Sys s = make_sys(d);
    if (alphaL > 0) s.alphaL = alphaL;
    if (kmax > 0) s.kmax = kmax;
    std::vector<V3> r = load_cfg(pos, s.N);
    return heg_ewald(s, r);
}

}  // extern "C"

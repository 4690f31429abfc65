// qmc_warp_kernels.cuh -- warp-per-walker kernels for systems with large spin
// sectors (benzene: 21x21 determinants, 42 electrons, 36 Gaussian AOs).
//
// One warp owns one walker.  Lane j holds column j of each inverse Slater
// matrix in registers (Dinv[k][j], k = 0..n-1) and the positions of
// electrons j and j+32.  AOs are evaluated lane-parallel from tables in
// shared memory; the AO->MO contraction, the determinant ratio and the
// Sherman-Morrison update broadcast one lane's values with shuffles, so every
// register index stays static.  The FP64 refresh is a warp-cooperative
// Gauss-Jordan elimination in which lane j carries column j of [D | I] and
// ends holding column j of D^-1 -- exactly the sweep kernel's layout.
#pragma once
#include <cstdio>
#include <cstring>
#include <vector>
#include "qmc_internal.h"
#include "qmc_device.cuh"

namespace qmc {

constexpr int WMAX_AO = 96;       // up to three rounds of 32 AOs (BenzeneGTO's 6-31G basis has 66)
constexpr int WAO_ROUNDS = WMAX_AO / 32;
constexpr int WNCOL = 24;         // Slater columns held per sector (lanes >= WNCOL read no coefficients)
constexpr int AO_REP = 16;        // ao_type flag: radial part equal to the previous AO's
constexpr int WMAX_PRIM = 256;
constexpr int WMAX_NUC = 16;

// Radial-group descriptor: nucleus (bits 0-3), kind (bit 4: 0 s, 1 p triplet),
// primitive count (bits 5-8), first primitive (bits 9-16), first AO (bits 17-23).
__host__ __device__ constexpr int grp_pack(int nuc, int kind, int np, int p0, int a0) {
    return nuc | (kind << 4) | (np << 5) | (p0 << 9) | (a0 << 17);
}
__host__ __device__ constexpr int grp_a0(int g) { return (g >> 17) & 127; }
static_assert(WMAX_NUC <= 16 && WMAX_PRIM <= 256 && WMAX_AO <= 128, "group descriptor fields");

// Shared-memory system table of the warp kernels (one copy per block).
template <class T>
struct SysW {
    int n_ao;
    int quirk_lap;
    T F, invF, qa, v_nn;
    T b_ee[2], a_ee[2];
    T nuc[WMAX_NUC][3];
    T Z[WMAX_NUC], enA[WMAX_NUC], enB[WMAX_NUC];
    // ao_type: bits 0-3 the kind (0 s, 1..3 p_x..p_z); AO_REP set when the AO has the
    // centre and primitives of the previous AO (p_y and p_z after p_x share its radial part)
    int ao_nuc[WMAX_AO], ao_type[WMAX_AO], ao_p0[WMAX_AO], ao_np[WMAX_AO];
    // radial groups in AO order: an s AO alone, or a p triplet sharing one
    // radial part; packed by grp_pack (nucleus, kind, primitives, first AO)
    int n_grp;
    int grp[WMAX_AO];
    alignas(16) T prim[WMAX_PRIM][2];   // (exponent, coefficient) of every primitive
    alignas(16) T C[2][WMAX_AO][WNCOL];     // [sector][AO][column]; 16-byte rows of 4 columns read as vectors
    T init_sigma;
    int init_nuc[64];           // internal electron order
    int perm[64];
};

template <class T>
static bool fill_sysw(const HostSys& hs, int NE, int NUP, int NNUC, SysW<T>& S) {
    std::memset(&S, 0, sizeof(S));
    if (hs.N != NE || hs.n_up != NUP || hs.n_nuc != NNUC || hs.n_ao > WMAX_AO || NNUC > WMAX_NUC) return false;
    if (NUP > WNCOL || NE - NUP > WNCOL) return false;
    if (hs.basis != BASIS_GTO) return false;
    S.n_ao = hs.n_ao;
    S.quirk_lap = (hs.quirks & 2) ? 1 : 0;
    S.F = (T)hs.F;
    S.invF = (T)(1.0 / hs.F);
    S.qa = (hs.quirks & 1) ? (T)hs.F : (T)1;
    S.v_nn = (T)hs.v_nn;
    S.b_ee[0] = (T)hs.jas[0]; S.b_ee[1] = (T)hs.jas[1];
    S.a_ee[0] = (T)hs.jas[2]; S.a_ee[1] = (T)hs.jas[3];
    for (int I = 0; I < NNUC; ++I) {
        for (int c = 0; c < 3; ++c) S.nuc[I][c] = (T)hs.R[3 * I + c];
        S.Z[I] = (T)hs.Z[I];
        int sp = hs.species[I];
        S.enA[I] = (T)(hs.jas[6 + sp] * hs.Z[I]);
        S.enB[I] = (T)hs.jas[4 + sp];
    }
    // AOs in internal (shell) order; each AO keeps its own primitive list
    int np = 0;
    for (const HostShell& sh : hs.shells) {
        auto put = [&](int caller_ao, int type, const std::vector<double>& coef) -> bool {
            int a = hs.ao_int[caller_ao];
            if ((int)(np + sh.exps.size()) > WMAX_PRIM || sh.exps.size() > 15) return false;
            S.ao_nuc[a] = sh.nuc;
            S.ao_type[a] = type;
            S.ao_p0[a] = np;
            S.ao_np[a] = (int)sh.exps.size();
            for (size_t p = 0; p < sh.exps.size(); ++p) { S.prim[np][0] = (T)sh.exps[p]; S.prim[np][1] = (T)coef[p]; ++np; }
            return true;
        };
        for (int k = 0; k < 2; ++k) {
            if (sh.s_ao[k] < 0) continue;
            const int p0 = np;
            if (!put(sh.s_ao[k], 0, sh.s_coef[k])) return false;
            S.grp[S.n_grp++] = grp_pack(sh.nuc, 0, (int)sh.exps.size(), p0, hs.ao_int[sh.s_ao[k]]);
        }
        // the p triplet's members are consecutive in the internal order and share
        // one radial part: p_y and p_z reuse p_x's
        if (sh.p_ao[0] >= 0) {
            const int p0 = np, a0 = hs.ao_int[sh.p_ao[0]];
            for (int m = 0; m < 3; ++m) {
                if (hs.ao_int[sh.p_ao[m]] != a0 + m) return false;
                if (!put(sh.p_ao[m], (1 + m) | (m > 0 ? AO_REP : 0), sh.p_coef)) return false;
            }
            S.grp[S.n_grp++] = grp_pack(sh.nuc, 1, (int)sh.exps.size(), p0, a0);
        }
    }
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
    S.init_sigma = (T)hs.init_sigma;
    for (int ei = 0; ei < hs.N; ++ei) {
        S.perm[ei] = hs.perm[ei];
        S.init_nuc[ei] = hs.init_nuc[hs.perm[ei]];
    }
    return true;
}

// Copy the table from global to shared memory (whole block).
template <class T>
__device__ __forceinline__ void load_sysw(SysW<T>* dst, const SysW<T>* __restrict__ src) {
    static_assert(sizeof(SysW<T>) % 4 == 0, "table size must be a multiple of 4 bytes");
    const int4* s = reinterpret_cast<const int4*>(src);
    int4* d = reinterpret_cast<int4*>(dst);
    constexpr int n16 = (int)(sizeof(SysW<T>) / sizeof(int4));
    for (int i = threadIdx.x; i < n16; i += blockDim.x) d[i] = s[i];
    // tail words when the size is not a multiple of 16 bytes
    for (int i = n16 * 4 + threadIdx.x; i < (int)(sizeof(SysW<T>) / 4); i += blockDim.x)
        reinterpret_cast<int*>(dst)[i] = reinterpret_cast<const int*>(src)[i];
    __syncthreads();
}

// (exponent, coefficient) pair of a primitive: one 8- or 16-byte shared load.
template <class T>
__device__ __forceinline__ void load2(const T (&p)[2], T& a, T& b) { a = p[0]; b = p[1]; }
__device__ __forceinline__ void load2(const float (&p)[2], float& a, float& b) {
    const float2 v = *reinterpret_cast<const float2*>(p);
    a = v.x; b = v.y;
}
__device__ __forceinline__ void load2(const double (&p)[2], double& a, double& b) {
    const double2 v = *reinterpret_cast<const double2*>(p);
    a = v.x; b = v.y;
}

// ---------------------------------------------------------------------------
// Lane-parallel AO evaluation: lane l evaluates AO l + 32 r in round r at
// point (x,y,z): value, gradient, Laplacian (MODE >= 1 / 2).  Rounds past the
// basis are skipped (a warp-uniform branch).
// ---------------------------------------------------------------------------
template <class T, int MODE>
struct AOLane {
    T v[WAO_ROUNDS], gx[WAO_ROUNDS], gy[WAO_ROUNDS], gz[WAO_ROUNDS], l[WAO_ROUNDS];
};

template <class T, int MODE>
__device__ __forceinline__ void ao_lane(const SysW<T>& S, T x, T y, T z, int lane, AOLane<T, MODE>& o) {
#pragma unroll
    for (int r = 0; r < WAO_ROUNDS; ++r) {
        const int a = lane + 32 * r;
        T v = 0, gxx = 0, gyy = 0, gzz = 0, lp = 0;
        if (32 * r < S.n_ao && a < S.n_ao) {
            const int I = S.ao_nuc[a], type = S.ao_type[a] & 15, p0 = S.ao_p0[a], np = S.ao_np[a];
            T dx = x - S.nuc[I][0], dy = y - S.nuc[I][1], dz = z - S.nuc[I][2];
            T r2 = dx * dx + dy * dy + dz * dz;
            T s0 = 0, s1 = 0, s2 = 0;
            for (int p = p0; p < p0 + np; ++p) {
                T al, cp;
                load2(S.prim[p], al, cp);
                T e = cp * fexp(-al * r2);
                s0 += e;
                if (MODE >= 1) s1 += al * e;
                if (MODE >= 2) s2 += al * al * e;
            }
            // s: chi = R; grad = -2 R1 dr; lap = -6 R1 + 4 r^2 R2
            // p_m: chi = x_m R; grad = x_m(-2 R1 dr) + e_m R; lap = x_m(-10 R1 + 4 r^2 R2)
            T ang = type == 0 ? T(1) : (type == 1 ? dx : (type == 2 ? dy : dz));
            v = ang * s0;
            if (MODE >= 1) {
                T g = -2 * s1 * ang;
                gxx = g * dx + (type == 1 ? s0 : T(0));
                gyy = g * dy + (type == 2 ? s0 : T(0));
                gzz = g * dz + (type == 3 ? s0 : T(0));
            }
            if (MODE >= 2) lp = ang * ((type == 0 ? T(-6) : T(-10)) * s1 + 4 * r2 * s2);
        }
        o.v[r] = v;
        if (MODE >= 1) { o.gx[r] = gxx; o.gy[r] = gyy; o.gz[r] = gzz; }
        if (MODE >= 2) o.l[r] = lp;
    }
}

__device__ __forceinline__ float wshfl(float v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ double wshfl(double v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ int wshfl(int v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ float wshfl_xor(float v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
__device__ __forceinline__ double wshfl_xor(double v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
__device__ __forceinline__ ff wshfl_xor(ff v, int m) { return shfl_xor(v, m); }
template <class T>
__device__ __forceinline__ T wsum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += wshfl_xor(v, o);
    return v;
}

// Four consecutive elements of 16-byte-aligned shared memory as one vector
// access (two for double).
__device__ __forceinline__ void load4(const float* p, float& a, float& b, float& c, float& d) {
    const float4 v = *reinterpret_cast<const float4*>(p);
    a = v.x; b = v.y; c = v.z; d = v.w;
}
__device__ __forceinline__ void load4(const double* p, double& a, double& b, double& c, double& d) {
    const double2 u = reinterpret_cast<const double2*>(p)[0], v = reinterpret_cast<const double2*>(p)[1];
    a = u.x; b = u.y; c = v.x; d = v.y;
}
__device__ __forceinline__ void store4(float* p, float a, float b, float c, float d) {
    *reinterpret_cast<float4*>(p) = make_float4(a, b, c, d);
}
__device__ __forceinline__ void store4(double* p, double a, double b, double c, double d) {
    reinterpret_cast<double2*>(p)[0] = make_double2(a, b);
    reinterpret_cast<double2*>(p)[1] = make_double2(c, d);
}

// Jastrow cache of the Gaussian sweep: u(r_ij) of every electron pair i < j
// at slot j (j - 1) / 2 + i, then the one-body sum U1_i = sum_I A_I Z_I r/(1 + B_I r)
// of every electron, rounded up to 4 elements.
template <int NE>
__host__ __device__ constexpr int jcache_elems() { return (NE * (NE - 1) / 2 + NE + 3) / 4 * 4; }
__device__ __forceinline__ int pair_slot(int i, int j) {
    const int a = i < j ? i : j, b = i < j ? j : i;
    return b * (b - 1) / 2 + a;
}

// Elements of the per-warp scratch of the single-electron sweep: one row of
// WNCOL orbital values per proposal of a sector, then the Jastrow cache.
template <int NE, int NUP>
__host__ __device__ constexpr int sweep_scratch_elems() {
    return (NUP > NE - NUP ? NUP : NE - NUP) * WNCOL + jcache_elems<NE>();
}

// MO contraction: lane k receives phi_k = sum_a C[sig][a][k] chi_a (and
// gradient / Laplacian), chi_a broadcast from lane a % 32; lanes past the
// table's columns accumulate zeros.
template <class T, int MODE>
__device__ __forceinline__ void mo_lane(const SysW<T>& S, int sig, int lane, const AOLane<T, MODE>& ao, T& v, T& gx,
                                        T& gy, T& gz, T& l) {
    v = 0; gx = 0; gy = 0; gz = 0; l = 0;
    const bool own = lane < WNCOL;
    const int col = own ? lane : 0;
#pragma unroll
    for (int r = 0; r < WAO_ROUNDS; ++r) {
        const int base = 32 * r;
        if (base >= S.n_ao) break;
        const int cnt = min(32, S.n_ao - base);
        for (int t = 0; t < cnt; ++t) {
            const T cl = S.C[sig][base + t][col];
            const T c = own ? cl : T(0);
            if (MODE != 3) v += c * wshfl(ao.v[r], t);
            if (MODE >= 1) {
                gx += c * wshfl(ao.gx[r], t);
                gy += c * wshfl(ao.gy[r], t);
                gz += c * wshfl(ao.gz[r], t);
            }
            if (MODE >= 2) l += c * wshfl(ao.l[r], t);
        }
    }
}

// c'_a = sum_k C[sig][a][k] Dinv[k][q] for the lane's AOs a = lane + 32 r: column q of
// the inverse (lane q's registers) broadcast four entries at a time, the lane's
// coefficient rows read as 16-byte vectors.  Lanes past the basis get 0.
template <class T, int NM>
__device__ __forceinline__ void inverse_column_coefficients(const SysW<T>& S, int sig, int lane, const T (&D)[NM],
                                                            int q, T (&cw)[WAO_ROUNDS]) {
#pragma unroll
    for (int r = 0; r < WAO_ROUNDS; ++r) cw[r] = 0;
#pragma unroll
    for (int k0 = 0; k0 < NM; k0 += 4) {
        T dq[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) dq[i] = (k0 + i < NM) ? wshfl(D[k0 + i < NM ? k0 + i : 0], q) : T(0);
#pragma unroll
        for (int r = 0; r < WAO_ROUNDS; ++r) {
            if (32 * r >= S.n_ao) break;
            const int a = lane + 32 * r;
            T c0, c1, c2, c3;
            load4(&S.C[sig][a < S.n_ao ? a : 0][k0], c0, c1, c2, c3);
            T t = c0 * dq[0] + c1 * dq[1] + c2 * dq[2] + c3 * dq[3];
            cw[r] += a < S.n_ao ? t : T(0);
        }
    }
}

// ---------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------
template <class TS>
__global__ void kw_init(const SysW<double>* __restrict__ Sg, TS* __restrict__ pos, int NE, int W, int Wcap,
                        uint64_t seed) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= NE * W) return;
    int e = i / W, w = i - e * W;
    const SysW<double>& S = *Sg;
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

// Positions of electrons `lane` and `lane + 32` live in this lane.
template <class T, int NE>
struct LanePos {
    T x[2], y[2], z[2];
    __device__ __forceinline__ void get(int e, T& ex, T& ey, T& ez) const {
        T a = e < 32 ? x[0] : x[1], b = e < 32 ? y[0] : y[1], c = e < 32 ? z[0] : z[1];
        ex = wshfl(a, e & 31); ey = wshfl(b, e & 31); ez = wshfl(c, e & 31);
    }
    // Same, for an index that differs between lanes: the source lane cannot know which
    // half the reading lane wants, so both halves travel and the reader selects.
    __device__ __forceinline__ void get_own(int e, T& ex, T& ey, T& ez) const {
        const int s = e & 31;
        T x0 = wshfl(x[0], s), x1 = wshfl(x[1], s), y0 = wshfl(y[0], s), y1 = wshfl(y[1], s);
        T z0 = wshfl(z[0], s), z1 = wshfl(z[1], s);
        ex = e < 32 ? x0 : x1; ey = e < 32 ? y0 : y1; ez = e < 32 ? z0 : z1;
    }
};

// This lane's share of the Jastrow terms of electron e at (x, y, z): u =
// sum_j u_ee(r_ej) - sum_I u_en(r_eI) and its gradient with respect to the
// electron, over partner electron `lane` (first round) and partner electron
// 32 + lane (lanes < NE1) or nucleus lane - NE1 (the next NNUC lanes; second
// round).  Every lane evaluates and the unused terms are masked by selects.
template <int NE, int NUP, int NNUC, class T>
__device__ __forceinline__ void wjastrow_lane_terms(const SysW<T>& S, const LanePos<T, NE>& P, int lane, int e,
                                                    T x, T y, T z, T& u, T (&g)[3]) {
    constexpr int NE1 = NE > 32 ? NE - 32 : 0;
    static_assert(NE <= 64 && NE1 + NNUC <= 32, "second round: electrons 32.. and the nuclei share the lanes");
    const bool e_up = e < NUP;
    {
        const int j = lane < NE ? lane : NE - 1;
        const bool ok = lane < NE && lane != e;
        const int c = ((j < NUP) == e_up) ? 1 : 0;
        const T dx = x - P.x[0], dy = y - P.y[0], dz = z - P.z[0];
        T d, ri, uu, upr, lt;
        dist(dx * dx + dy * dy + dz * dz, d, ri);
        pade_ab(S.a_ee[c], S.b_ee[c], d, ri, uu, upr, lt);
        u = ok ? uu : T(0);
        const T f = ok ? upr : T(0);
        g[0] = f * dx; g[1] = f * dy; g[2] = f * dz;
    }
    {
        const bool is_el = lane < NE1, is_nuc = !is_el && lane - NE1 < NNUC;
        const int j = is_el ? 32 + lane : 0, I = is_nuc ? lane - NE1 : 0;
        const bool el_ok = is_el && j != e;
        const T ox = is_el ? P.x[1] : S.nuc[I][0], oy = is_el ? P.y[1] : S.nuc[I][1];
        const T oz = is_el ? P.z[1] : S.nuc[I][2];
        const int c = ((j < NUP) == e_up) ? 1 : 0;
        const T pa = is_el ? S.a_ee[c] : S.enA[I], pb = is_el ? S.b_ee[c] : S.enB[I];
        const T dx = x - ox, dy = y - oy, dz = z - oz;
        T d, ri, uu, upr, lt;
        dist(dx * dx + dy * dy + dz * dz, d, ri);
        pade_ab(pa, pb, d, ri, uu, upr, lt);
        u += el_ok ? uu : (is_nuc ? -uu : T(0));
        const T f = el_ok ? upr : (is_nuc ? -upr : T(0));
        g[0] += f * dx; g[1] += f * dy; g[2] += f * dz;
    }
}

// Row stride of the per-warp proposal-orbital scratch (a multiple of 4
// elements, so that rows start 16-byte aligned and read as vectors).
constexpr int PHS = WNCOL;

// acc[k] += c[k] chi for k < NM: coefficient rows are read as 16-byte vectors
// (NM / 4 of them) and NM % 4 scalars, so no padding column is multiplied.
template <class T, int NM>
__device__ __forceinline__ void row_axpy(const T* c, T chi, T (&acc)[NM]) {
#pragma unroll
    for (int v = 0; v < NM / 4; ++v) {
        T c0, c1, c2, c3;
        load4(c + 4 * v, c0, c1, c2, c3);
        acc[4 * v + 0] += c0 * chi; acc[4 * v + 1] += c1 * chi;
        acc[4 * v + 2] += c2 * chi; acc[4 * v + 3] += c3 * chi;
    }
#pragma unroll
    for (int k = 4 * (NM / 4); k < NM; ++k) acc[k] += c[k] * chi;
}

// Orbital values phi_k(x, y, z), k < NM, of sector sig by one lane: one pass
// over the radial groups (an s AO, or a p triplet sharing its radial part),
// each contracted into the table's columns (broadcast reads: every lane reads
// the same coefficients); written to out[k].
template <class T, int NM>
__device__ __forceinline__ void proposal_orbitals(const SysW<T>& S, int sig, T x, T y, T z, T* out) {
    T acc[NM];
#pragma unroll
    for (int k = 0; k < NM; ++k) acc[k] = 0;
    for (int g = 0; g < S.n_grp; ++g) {
        const int d = S.grp[g];
        const int I = d & 15, kind = (d >> 4) & 1, np = (d >> 5) & 15, p0 = (d >> 9) & 255, a0 = grp_a0(d);
        const T dx = x - S.nuc[I][0], dy = y - S.nuc[I][1], dz = z - S.nuc[I][2];
        const T r2 = dx * dx + dy * dy + dz * dz;
        T s0 = 0;
        for (int p = p0; p < p0 + np; ++p) {
            T al, cp;
            load2(S.prim[p], al, cp);
            s0 += cp * fexp(-al * r2);
        }
        const T* c = S.C[sig][a0];
        if (kind == 0) {
            row_axpy<T, NM>(c, s0, acc);
        } else {
            row_axpy<T, NM>(c, dx * s0, acc);
            row_axpy<T, NM>(c + WNCOL, dy * s0, acc);
            row_axpy<T, NM>(c + 2 * WNCOL, dz * s0, acc);
        }
    }
#pragma unroll
    for (int v = 0; v < NM / 4; ++v) store4(out + 4 * v, acc[4 * v], acc[4 * v + 1], acc[4 * v + 2], acc[4 * v + 3]);
#pragma unroll
    for (int k = 4 * (NM / 4); k < NM; ++k) out[k] = acc[k];
}

// Single-electron sweeps, one warp per walker, WPB walkers per block.  A is
// const SweepArgs<T> or const volatile SweepArgs<T>.  Gaussian moves take a
// sector's proposals together: an electron of the sector keeps its position
// until its own proposal, so all NS proposed positions are known when the
// sector's turn starts; lane i evaluates the orbitals at proposal i into the
// warp's scratch ph (proposal_orbitals), and each proposal then reads its row
// as a broadcast instead of contracting AO values broadcast lane to lane.
// Drift-diffusion proposals depend on the current drift and stay one at a
// time.
template <int NE, int NUP, int NNUC, class T, int MOVE, class A>
__device__ __forceinline__ void kw_sweep_walker(const SysW<T>& S, A& a, int w, T* ph) {
    constexpr int NDN = NE - NUP;
    constexpr int NM = NUP > NDN ? NUP : NDN;
    constexpr int NE1 = NE > 32 ? NE - 32 : 0;   // partner electrons of the second round
    static_assert(NE <= 64 && NE1 + NNUC <= 32, "second round: electrons 32.. and the nuclei share the lanes");
    const int lane = threadIdx.x & 31;
    LanePos<T, NE> P;
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        const int j = lane + 32 * r;
        const bool ok = j < NE;
        P.x[r] = ok ? a.pos[(3 * j + 0) * (size_t)a.Wcap + w] : T(0);
        P.y[r] = ok ? a.pos[(3 * j + 1) * (size_t)a.Wcap + w] : T(0);
        P.z[r] = ok ? a.pos[(3 * j + 2) * (size_t)a.Wcap + w] : T(0);
    }
    T D0[NM], D1[NM];
#pragma unroll
    for (int k = 0; k < NM; ++k) {
        D0[k] = lane < NUP ? a.dinv[((size_t)(0 * NM * NM + k * NM + lane)) * a.Wcap + w] : T(0);
        D1[k] = lane < NDN ? a.dinv[((size_t)(1 * NM * NM + k * NM + lane)) * a.Wcap + w] : T(0);
    }
    int sgn = a.sign[w];
    unsigned acc = 0;
    int flg = 0;
    // Gaussian moves keep every pair term and every one-body sum in the
    // warp's cache (jc), so a proposal evaluates only the moving electron's
    // new terms; a cached term is the same expression on the same squared
    // distance as a recomputation, hence the same value.
    constexpr int NPAIR = NE * (NE - 1) / 2;
    T* jc = ph + NM * PHS;
    if constexpr (MOVE == MOVE_ONE_GAUSS) {
        for (int i = 0; i < NE; ++i) {
            T xi, yi, zi;
            P.get(i, xi, yi, zi);
#pragma unroll
            for (int r = 0; r < 2; ++r) {
                const int j = lane + 32 * r;
                if (j < NE && j > i) {
                    T dx = xi - (r ? P.x[1] : P.x[0]), dy = yi - (r ? P.y[1] : P.y[0]), dz = zi - (r ? P.z[1] : P.z[0]);
                    T d, ri, uu, upr, lt;
                    dist(dx * dx + dy * dy + dz * dz, d, ri);
                    const int c = ((j < NUP) == (i < NUP)) ? 1 : 0;
                    pade_ab(S.a_ee[c], S.b_ee[c], d, ri, uu, upr, lt);
                    jc[pair_slot(i, j)] = uu;
                }
            }
            T en = 0;
            if (lane < NNUC) {
                T dx = xi - S.nuc[lane][0], dy = yi - S.nuc[lane][1], dz = zi - S.nuc[lane][2];
                T d, ri, uu, upr, lt;
                dist(dx * dx + dy * dy + dz * dz, d, ri);
                pade_ab(S.enA[lane], S.enB[lane], d, ri, uu, upr, lt);
                en = uu;
            }
            en = wsum(en);
            if (lane == 0) jc[NPAIR + i] = en;
        }
        __syncwarp();
    }
    for (int it = 0; it < a.n_sweeps; ++it) {
        const uint64_t st = a.step0 + (uint64_t)it;
#pragma unroll
        for (int sig = 0; sig < 2; ++sig) {
            T (&D)[NM] = sig == 0 ? D0 : D1;
            const int NS = sig == 0 ? NUP : NDN;
            static_assert(NUP <= 32 && NE - NUP <= 32, "one lane per sector electron");
            const MoveDraw<T> draws = sector_draws<T>(a.seed, (uint32_t)w, st, sig * NUP, NS, lane);
            T pnx = 0, pny = 0, pnz = 0;              // this lane's proposal (Gaussian moves)
            if constexpr (MOVE == MOVE_ONE_GAUSS) {
                T ex, ey, ez;
                P.get_own(min(sig * NUP + lane, NE - 1), ex, ey, ez);
                const T step = a.step;
                pnx = ex + step * draws.n0; pny = ey + step * draws.n1; pnz = ez + step * draws.n2;
                __syncwarp();                          // the previous sector's rows are read
                if (lane < NS) proposal_orbitals<T, NM>(S, sig, pnx, pny, pnz, ph + lane * PHS);
                __syncwarp();
            }
            T csc = 1;                                 // pending scale of this lane's column (Gaussian moves)
            for (int q = 0; q < NS; ++q) {
                const int e = sig * NUP + q;
                T rx, ry, rz;
                P.get(e, rx, ry, rz);
                const MoveDraw<T> md = draw_of(draws, q);
                T nx, ny, nz, logG = 0, dlx = 0, dly = 0, dlz = 0;
                // drift: c'_a = sum_k C[sig][a][k] Dinv[k][q] on the lanes of AO a, so that
                // grad ln D at r and at r' are sums over the AOs (warp sums)
                T cw[WAO_ROUNDS];
                T u_old = 0;                           // drift: this lane's Jastrow terms at r
                if constexpr (MOVE == MOVE_ONE_DRIFT) {
                    inverse_column_coefficients<T, NM>(S, sig, lane, D, q, cw);
                    AOLane<T, 1> ao;
                    ao_lane<T, 1>(S, rx, ry, rz, lane, ao);
                    T ax = 0, ay = 0, az = 0;
#pragma unroll
                    for (int r = 0; r < WAO_ROUNDS; ++r) { ax += cw[r] * ao.gx[r]; ay += cw[r] * ao.gy[r]; az += cw[r] * ao.gz[r]; }
                    ax = wsum(ax); ay = wsum(ay); az = wsum(az);
                    T gl[3];
                    wjastrow_lane_terms<NE, NUP, NNUC, T>(S, P, lane, e, rx, ry, rz, u_old, gl);
                    T g0[3];
#pragma unroll
                    for (int c = 0; c < 3; ++c) g0[c] = wsum(gl[c]) * S.qa;
                    const T tau = a.tau, maxd = a.maxd;
                    dlx = tau * 2 * (ax + g0[0]); dly = tau * 2 * (ay + g0[1]); dlz = tau * 2 * (az + g0[2]);
                    T m = fsqrt(dlx * dlx + dly * dly + dlz * dlz);
                    if (m > maxd) { T s = maxd / m; dlx *= s; dly *= s; dlz *= s; }
                    T sd2 = fsqrt(2 * tau);
                    nx = rx + dlx + sd2 * md.n0; ny = ry + dly + sd2 * md.n1; nz = rz + dlz + sd2 * md.n2;
                } else {
                    nx = wshfl(pnx, q); ny = wshfl(pny, q); nz = wshfl(pnz, q);
                }
                // t_j = sum_k phi_k Dinv[k][j]; R = t_q
                T tj = 0, bx = 0, by = 0, bz = 0;
                if constexpr (MOVE == MOVE_ONE_DRIFT) {
                    AOLane<T, 1> ao;
                    ao_lane<T, 1>(S, nx, ny, nz, lane, ao);
                    // orbital values at r' (every t_j is needed for the update), the
                    // gradient term of column q from c'
                    AOLane<T, 0> av;
#pragma unroll
                    for (int r = 0; r < WAO_ROUNDS; ++r) av.v[r] = ao.v[r];
                    T phi, pgx, pgy, pgz, pl;
                    mo_lane<T, 0>(S, sig, lane, av, phi, pgx, pgy, pgz, pl);
#pragma unroll
                    for (int k = 0; k < NM; ++k) tj += wshfl(phi, k) * D[k];
#pragma unroll
                    for (int r = 0; r < WAO_ROUNDS; ++r) { bx += cw[r] * ao.gx[r]; by += cw[r] * ao.gy[r]; bz += cw[r] * ao.gz[r]; }
                    bx = wsum(bx); by = wsum(by); bz = wsum(bz);
                } else {
                    const T* row = ph + q * PHS;
                    T t0 = 0, t1 = 0;
#pragma unroll
                    for (int v = 0; v < (NM + 3) / 4; ++v) {
                        T f0, f1, f2, f3;
                        load4(row + 4 * v, f0, f1, f2, f3);
                        if (4 * v + 0 < NM) t0 += f0 * D[4 * v + 0];
                        if (4 * v + 1 < NM) t1 += f1 * D[4 * v + 1];
                        if (4 * v + 2 < NM) t0 += f2 * D[4 * v + 2];
                        if (4 * v + 3 < NM) t1 += f3 * D[4 * v + 3];
                    }
                    tj = t0 + t1;
                }
                const T R = wshfl(tj, q);
                T gn[3];
                T du, unew[2] = {T(0), T(0)}, enn = 0;
                if constexpr (MOVE == MOVE_ONE_GAUSS) {
                    // new terms of the moving electron against the cached old
                    // ones: partner electron `lane` in the first round; in the
                    // second, partner electron 32 + lane on lanes < NE1 and
                    // nucleus lane - NE1 on the next NNUC lanes
                    // Every lane evaluates its terms and the unused ones are
                    // masked out (no divergent branch; the masked lanes read a
                    // valid cache slot and may compute non-finite values).
                    T ds;
                    {
                        const int j = lane < NE ? lane : NE - 1;
                        T dx = nx - P.x[0], dy = ny - P.y[0], dz = nz - P.z[0];
                        T d, ri, uu, upr, lt;
                        dist(dx * dx + dy * dy + dz * dz, d, ri);
                        const int c = ((j < NUP) == (e < NUP)) ? 1 : 0;
                        pade_ab(S.a_ee[c], S.b_ee[c], d, ri, uu, upr, lt);
                        unew[0] = uu;
                        const T old = jc[pair_slot(e, j)];
                        ds = (lane < NE && lane != e) ? uu - old : T(0);
                    }
                    {
                        const bool is_el = lane < NE1, is_nuc = !is_el && lane - NE1 < NNUC;
                        const int j = is_el ? 32 + lane : 0, I = is_nuc ? lane - NE1 : 0;
                        const T ox = is_el ? P.x[1] : S.nuc[I][0], oy = is_el ? P.y[1] : S.nuc[I][1];
                        const T oz = is_el ? P.z[1] : S.nuc[I][2];
                        const int c = ((j < NUP) == (e < NUP)) ? 1 : 0;
                        const T pa = is_el ? S.a_ee[c] : S.enA[I], pb = is_el ? S.b_ee[c] : S.enB[I];
                        T dx = nx - ox, dy = ny - oy, dz = nz - oz;
                        T d, ri, uu, upr, lt;
                        dist(dx * dx + dy * dy + dz * dz, d, ri);
                        pade_ab(pa, pb, d, ri, uu, upr, lt);
                        unew[1] = uu;
                        const T old = jc[pair_slot(e, j)];
                        ds += (is_el && j != e) ? uu - old : T(0);
                        enn = is_nuc ? uu : T(0);
                        ds -= enn;
                    }
                    du = wsum(ds) + jc[NPAIR + e];
                } else {
                    // new position's terms against the old position's (kept from the drift)
                    T un, gl[3];
                    wjastrow_lane_terms<NE, NUP, NNUC, T>(S, P, lane, e, nx, ny, nz, un, gl);
                    du = wsum(un - u_old);
#pragma unroll
                    for (int c = 0; c < 3; ++c) gn[c] = wsum(gl[c]) * S.qa;
                }
                if constexpr (MOVE == MOVE_ONE_DRIFT) {
                    const T tau = a.tau, maxd = a.maxd;
                    T iR = R != T(0) ? T(1) / R : T(0);
                    T cx = tau * 2 * (bx * iR + gn[0]), cy = tau * 2 * (by * iR + gn[1]), cz = tau * 2 * (bz * iR + gn[2]);
                    T m = fsqrt(cx * cx + cy * cy + cz * cz);
                    if (m > maxd) { T s = maxd / m; cx *= s; cy *= s; cz *= s; }
                    T fx = nx - rx - dlx, fy = ny - ry - dly, fz = nz - rz - dlz;
                    T qx = rx - nx - cx, qy = ry - ny - cy, qz = rz - nz - cz;
                    logG = ((fx * fx + fy * fy + fz * fz) - (qx * qx + qy * qy + qz * qz)) / (4 * tau);
                }
                T ratio = R * fexp(du);
                T prob = ratio * ratio;
                if (MOVE == MOVE_ONE_DRIFT) prob *= fexp(logG);
                if (prob != prob) flg |= FLAG_NONFINITE;
                if (md.uacc < prob && R != T(0) && !(a.fixed_node && R < T(0))) {
                    // positions: the owner lane of e stores the new coordinates
                    if ((e & 31) == lane) {
                        if (e < 32) { P.x[0] = nx; P.y[0] = ny; P.z[0] = nz; }
                        else { P.x[1] = nx; P.y[1] = ny; P.z[1] = nz; }
                    }
                    const T iR = T(1) / R;
                    if constexpr (MOVE == MOVE_ONE_GAUSS) {
                        // column q keeps its values and takes the factor 1/R,
                        // applied when the sector ends (every column's scale is
                        // 1 until its own electron moves, so t_q and R are read
                        // unscaled); the others take t_j / R times column q
                        const T f = lane == q ? T(0) : tj * iR;
                        if (lane == q) csc = iR;
#pragma unroll
                        for (int k = 0; k < NM; ++k) D[k] -= wshfl(D[k], q) * f;
                    } else {
                        const T f = tj * iR;
#pragma unroll
                        for (int k = 0; k < NM; ++k) {
                            T dq = wshfl(D[k], q);
                            D[k] = (lane == q) ? dq * iR : D[k] - dq * f;
                        }
                    }
                    if (R < 0) sgn = -sgn;
                    ++acc;
                    if constexpr (MOVE == MOVE_ONE_GAUSS) {
                        if (lane < NE && lane != e) jc[pair_slot(e, lane)] = unew[0];
                        if (lane < NE1 && 32 + lane != e) jc[pair_slot(e, 32 + lane)] = unew[1];
                        const T u1 = wsum(enn);
                        if (lane == 0) jc[NPAIR + e] = u1;
                    }
                }
                __syncwarp();                      // cache writes before the next proposal's reads
            }
            if constexpr (MOVE == MOVE_ONE_GAUSS) {
#pragma unroll
                for (int k = 0; k < NM; ++k) D[k] *= csc;
            }
        }
    }
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        const int j = lane + 32 * r;
        if (j < NE) {
            a.pos[(3 * j + 0) * (size_t)a.Wcap + w] = P.x[r];
            a.pos[(3 * j + 1) * (size_t)a.Wcap + w] = P.y[r];
            a.pos[(3 * j + 2) * (size_t)a.Wcap + w] = P.z[r];
        }
    }
#pragma unroll
    for (int k = 0; k < NM; ++k) {
        if (lane < NUP) a.dinv[((size_t)(0 * NM * NM + k * NM + lane)) * a.Wcap + w] = D0[k];
        if (lane < NDN) a.dinv[((size_t)(1 * NM * NM + k * NM + lane)) * a.Wcap + w] = D1[k];
    }
    if (lane == 0) {
        a.sign[w] = sgn;
        if (acc) atomicAdd(a.acc, (unsigned long long)acc);
        if (flg) atomicOr(a.flags, flg);
    }
}

// FP32: four 4-walker blocks per SM (<= 128 registers)
template <int NE, int NUP, int NNUC, class T, int MOVE, int WPB>
__global__ void __launch_bounds__(32 * WPB, sizeof(T) == 4 ? 16 / WPB : 1) kw_sweep(const SysW<T>* __restrict__ Sg, T* __restrict__ gpos,
                                                     T* __restrict__ gdinv, int* __restrict__ gsign, int W, int Wcap,
                                                     int n_sweeps, uint64_t step0, T step, T tau, T maxd,
                                                     uint64_t seed, unsigned long long* acc_out, int* flags,
                                                     int fixed_node) {
    __shared__ SysW<T> S;
    __shared__ SweepArgs<T> args;
    if (threadIdx.x == 0)
        args = SweepArgs<T>{gpos, gdinv, gsign, acc_out, flags, step0, seed, step, tau, maxd, W, Wcap, n_sweeps,
                            fixed_node};
    extern __shared__ __align__(16) unsigned char wsm[];
    load_sysw(&S, Sg);                         // ends with a block barrier
    const int w = blockIdx.x * WPB + (threadIdx.x >> 5);
    if (w >= W) return;                        // whole warps only; no block barrier below
    const volatile SweepArgs<T>& a = args;
    T* ph = reinterpret_cast<T*>(wsm) + (size_t)(threadIdx.x >> 5) * sweep_scratch_elems<NE, NUP>();
    kw_sweep_walker<NE, NUP, NNUC, T, MOVE>(S, a, w, ph);
}

// Batched form: TW / WPB blocks per (system, TW-walker tile), each sweeping
// WPB walkers of it.  The hardware block scheduler balances uneven systems
// and classes that run side by side, and the kernel carries no tile-loop
// state into the walker's registers.
template <int NE, int NUP, int NNUC, class T, int MOVE, int WPB, int TW>
__global__ void __launch_bounds__(32 * WPB, sizeof(T) == 4 ? 16 / WPB : 1) kwb_sweep(const BatchTile* __restrict__ tiles, int ntiles,
                                                      const BatchRec* __restrict__ recs,
                                                      const BatchCtl* __restrict__ ctl) {
    static_assert(TW % WPB == 0, "a tile splits into whole blocks");
    constexpr int BPT = TW / WPB;
    __shared__ SysW<T> S;
    __shared__ SweepArgs<T> args;
    if ((int)blockIdx.x >= ntiles * BPT) return;
    const BatchTile tl = tiles[blockIdx.x / BPT];
    if (threadIdx.x == 0) args = sweep_args<T>(recs[tl.rec], *ctl);
    extern __shared__ __align__(16) unsigned char wsm[];
    load_sysw(&S, static_cast<const SysW<T>*>(recs[tl.rec].tab_s));   // ends with a block barrier
    const volatile SweepArgs<T>& a = args;
    const int w = tl.w0 + (int)(blockIdx.x % BPT) * WPB + (int)(threadIdx.x >> 5);
    if (w >= a.W) return;                      // whole warps only; no block barrier below
    T* ph = reinterpret_cast<T*>(wsm) + (size_t)(threadIdx.x >> 5) * sweep_scratch_elems<NE, NUP>();
    kw_sweep_walker<NE, NUP, NNUC, T, MOVE>(S, a, w, ph);
}

// Full evaluation from positions (refresh + E_L), one warp per walker.
// Per-warp shared scratch holds the sector's D rows, then the rows of its
// inverse; orbital derivatives are evaluated in a second pass.
// Row stride of the refresh's per-warp matrix scratch: lane q writes row q
// (element (q, k) at q MRS + k) and lane j reads column j; an odd stride keeps
// both conflict-free.
constexpr int MRS = 33;

// Orbital values phi_k(x, y, z), k < NM, of sector sig by one lane: one pass
// over the radial groups, lazily accumulated in the compute type.
template <class TC, int NM>
__device__ __forceinline__ void orbital_values(const SysW<TC>& S, int sig, TC x, TC y, TC z, TC (&v)[NM]) {
#pragma unroll
    for (int k = 0; k < NM; ++k) v[k] = 0;
    for (int g = 0; g < S.n_grp; ++g) {
        const int d = S.grp[g];
        const int I = d & 15, kind = (d >> 4) & 1, np = (d >> 5) & 15, p0 = (d >> 9) & 255, a0 = grp_a0(d);
        const TC dx = x - S.nuc[I][0], dy = y - S.nuc[I][1], dz = z - S.nuc[I][2];
        const TC r2 = dx * dx + dy * dy + dz * dz;
        TC s0 = 0;
        for (int p = p0; p < p0 + np; ++p) {
            TC al_p, cp;
            load2(S.prim[p], al_p, cp);
            s0 += cp * fexp(-al_p * r2);
        }
        for (int m = 0; m < (kind ? 3 : 1); ++m) {
            const TC chi = kind ? (m == 0 ? dx : (m == 1 ? dy : dz)) * s0 : s0;
            const TC* c = S.C[sig][a0 + m];
#pragma unroll
            for (int k = 0; k < NM; ++k) macc(v[k], c[k], chi);
        }
    }
#pragma unroll
    for (int k = 0; k < NM; ++k) v[k] = macc_norm(v[k]);
}

// sum_a c'_a (grad chi_a, lap chi_a) at (x, y, z) with c'_a = sum_k C[sig][a][k] dcol[k]:
// one pass over the radial groups (s AO, or p triplet sharing its radial part;
// s: grad = -2 R1 dr, lap = -6 R1 + 4 r^2 R2; p_m: grad = x_m (-2 R1 dr) + e_m R0,
// lap = x_m (-10 R1 + 4 r^2 R2), with R0, R1, R2 the radial sums weighted by
// 1, alpha, alpha^2).
template <class TC, int NM>
__device__ __forceinline__ void inverse_weighted_derivatives(const SysW<TC>& S, int sig, TC x, TC y, TC z,
                                                             const TC (&dcol)[NM], TC& gx, TC& gy, TC& gz, TC& lp) {
    TC ax = 0, ay = 0, az = 0, al = 0;
    for (int g = 0; g < S.n_grp; ++g) {
        const int d = S.grp[g];
        const int I = d & 15, kind = (d >> 4) & 1, np = (d >> 5) & 15, p0 = (d >> 9) & 255, a0 = grp_a0(d);
        const TC dx = x - S.nuc[I][0], dy = y - S.nuc[I][1], dz = z - S.nuc[I][2];
        const TC r2 = dx * dx + dy * dy + dz * dz;
        TC s0 = 0, s1 = 0, s2 = 0;
        for (int p = p0; p < p0 + np; ++p) {
            TC al_p, cp;
            load2(S.prim[p], al_p, cp);
            const TC e = cp * fexp(-al_p * r2), ea = al_p * e;
            s0 += e; s1 += ea; s2 += al_p * ea;
        }
        const TC l0 = TC(4) * r2 * s2;
        for (int m = 0; m < (kind ? 3 : 1); ++m) {
            const TC* c = S.C[sig][a0 + m];
            TC cw = 0;
#pragma unroll
            for (int k = 0; k < NM; ++k) macc(cw, c[k], dcol[k]);
            cw = macc_norm(cw);
            TC gxa, gya, gza, la;
            if (kind == 0) {
                const TC t = TC(-2) * s1;
                gxa = t * dx; gya = t * dy; gza = t * dz;
                la = TC(-6) * s1 + l0;
            } else {
                const TC xm = m == 0 ? dx : (m == 1 ? dy : dz);
                const TC t = TC(-2) * s1 * xm;
                gxa = t * dx + (m == 0 ? s0 : TC(0));
                gya = t * dy + (m == 1 ? s0 : TC(0));
                gza = t * dz + (m == 2 ? s0 : TC(0));
                la = xm * (TC(-10) * s1 + l0);
            }
            macc(ax, cw, gxa); macc(ay, cw, gya); macc(az, cw, gza); macc(al, cw, la);
        }
    }
    gx = macc_norm(ax); gy = macc_norm(ay); gz = macc_norm(az); lp = macc_norm(al);
}

template <int NE, int NUP, int NNUC, class TC, class TS>
__device__ __forceinline__ double kw_measure_walker(const SysW<TC>& S, TC* Mrow, const TS* __restrict__ gpos,
                                                    TS* __restrict__ gdinv, double* __restrict__ glog,
                                                    int* __restrict__ gsign, double* __restrict__ gel, int w,
                                                    bool act, int Wcap, int write_state,
                                                    double* __restrict__ out_grad, double* __restrict__ out_lap,
                                                    int* flags) {
    constexpr int NDN = NE - NUP;
    constexpr int NM = NUP > NDN ? NUP : NDN;
    const int lane = threadIdx.x & 31;
    double e_l = 0.0;
    if (act) {
        LanePos<TC, NE> P;
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            const int j = lane + 32 * r;
            const bool ok = j < NE;
            P.x[r] = ok ? (TC)gpos[(3 * j + 0) * (size_t)Wcap + w] : TC(0);
            P.y[r] = ok ? (TC)gpos[(3 * j + 1) * (size_t)Wcap + w] : TC(0);
            P.z[r] = ok ? (TC)gpos[(3 * j + 2) * (size_t)Wcap + w] : TC(0);
        }
        double logdet = 0.0;
        ff pmag = ff(1.0f);                       // float-float form: |det| = pmag 2^pexp
        int pexp = 0;
        int sg = 1;
        bool ok = true;
        // per-lane electron results: lane owns electron (sig*NUP + lane) of each sector
        TC gdx[2] = {0, 0}, gdy[2] = {0, 0}, gdz[2] = {0, 0}, ld[2] = {0, 0};
#pragma unroll
        for (int sig = 0; sig < 2; ++sig) {
            const int NS = sig == 0 ? NUP : NDN;
            // pass 1, lane q = electron q of the sector: its orbital values,
            // written as row q of D
            TC xq, yq, zq;
            P.get_own(min(sig * NUP + lane, NE - 1), xq, yq, zq);
            if (lane < NS) {
                TC v[NM];
                orbital_values<TC, NM>(S, sig, xq, yq, zq, v);
#pragma unroll
                for (int k = 0; k < NM; ++k)
                    if (k < NS) Mrow[lane * MRS + k] = v[k];
            }
            __syncwarp();
            // Gauss-Jordan in place with partial pivoting: lane j carries
            // column j of D and ends with column j of the inverse of the
            // row-permuted matrix.  Step k: rows k and p = argmax |D[i][k]|
            // interchanged; row k divided by a = D[k][k], column k becomes
            // -D[i][k]/a (1/a on the diagonal), the rest loses D[i][k] x row k
            // -- lane k's update takes the same form with t = 1 + 1/a.  The row
            // interchanges are undone as column interchanges: lane j gathers
            // column src(j), src = tau_{n-1}( ... tau_0(j)).  The pivot loop is
            // rolled, one copy of the step's code for all NS steps: the
            // registers hold the rows rotated so that row k sits in register 0
            // at step k (rows not yet pivoted first, in the order an unrolled
            // loop would have them), and each step moves register 0 to the back.
            TC A[NM];
#pragma unroll
            for (int i = 0; i < NM; ++i) A[i] = (i < NS && lane < NS) ? Mrow[i * MRS + lane] : TC(i == lane ? 1 : 0);
            int src = lane;
#pragma unroll 1
            for (int k = 0; k < NS; ++k) {
                int p = 0;
                float best = fabsf(lead(A[0]));
#pragma unroll
                for (int r = 1; r < NM; ++r) {
                    const float m = fabsf(lead(A[r]));
                    if (r < NS - k && m > best) { best = m; p = r; }
                }
                p = wshfl(p, k);
#pragma unroll
                for (int r = 1; r < NM; ++r) {
                    bool sw = (r == p);
                    TC a = A[0], b = A[r];
                    A[0] = sw ? b : a; A[r] = sw ? a : b;
                }
                if (p != 0) sg = -sg;
                const int pk = k + p;
                src = (src == k) ? pk : ((src == pk) ? k : src);
                TC piv = wshfl(A[0], k);
                if (!(piv != TC(0))) { ok = false; piv = TC(1); }
                if (piv < 0) sg = -sg;
                if constexpr (std::is_same<TC, ff>::value) {
                    pmag = pmag * fabs(piv);           // |det| as a rescaled product
                    ff_rescale(pmag, pexp);
                } else {
                    logdet += log(fabs((double)piv));
                }
                const TC ip = TC(1) / piv;
                const TC t = (lane == k) ? TC(1) + ip : A[0] * ip;
                A[0] = (lane == k) ? ip : t;
#pragma unroll
                for (int i = 1; i < NM; ++i) {
                    if (i >= NS) continue;
                    const TC f = wshfl(A[i], k);
                    A[i] -= f * t;
                }
                // rotate registers 0..NS-1 by one: the pivoted row goes last
                const TC r0 = A[0];
#pragma unroll
                for (int i = 0; i + 1 < NM; ++i) {
                    if (i + 1 < NS) A[i] = A[i + 1];
                    else if (i + 1 == NS) A[i] = r0;
                }
                if (NS == NM) A[NM - 1] = r0;
            }
            // unscramble: lane j takes column src(j); then A[k] = D^-1[k][lane]
#pragma unroll
            for (int i = 0; i < NM; ++i) {
                if (i >= NS) break;
                A[i] = wshfl(A[i], src);
            }
            if (write_state && lane < NS) {
#pragma unroll
                for (int k = 0; k < NM; ++k)
                    if (k < NS) gdinv[((size_t)(sig * NM * NM + k * NM + lane)) * Wcap + w] = (TS)A[k];
            }
            __syncwarp();
            // pass 2, lane q = electron q of the sector, holding column q of
            // D^-1: grad ln D = sum_k grad phi_k(r_q) D^-1[k][q] = sum_a c'_a
            // grad chi_a(r_q) with c'_a = sum_k C[a][k] D^-1[k][q] (the inverse
            // column contracted into the coefficients first), and the same for
            // lap D / D, over the radial groups at the lane's own electron
            if (lane < NS)
                inverse_weighted_derivatives<TC, NM>(S, sig, xq, yq, zq, A, gdx[sig], gdy[sig], gdz[sig], ld[sig]);
            __syncwarp();
        }
        // Jastrow + Coulomb for this lane's electrons (pairs counted from both ends)
        TC u = 0, V = 0, kin = 0;
#pragma unroll
        for (int sig = 0; sig < 2; ++sig) {
            const int NS = sig == 0 ? NUP : NDN;
            const int i = sig * NUP + lane;
            const bool own = lane < NS;
            TC xi, yi, zi;
            P.get_own(min(i, NE - 1), xi, yi, zi);
            TC gx = 0, gy = 0, gz = 0, lu = 0, gsq = 0;
            for (int j = 0; j < NE; ++j) {
                TC xj, yj, zj;
                P.get(j, xj, yj, zj);
                if (!own || j == i) continue;
                const bool para = ((j < NUP) == (i < NUP));
                TC dx = xi - xj, dy = yi - yj, dz = zi - zj;
                TC d, ri;
                dist(dx * dx + dy * dy + dz * dz, d, ri);
                V += TC(0.5) * ri;
                TC uu, upr, lt;
                const int c = para ? 1 : 0;
                pade_ab(S.a_ee[c], S.b_ee[c], d, ri, uu, upr, lt);
                u += TC(0.5) * uu;
                if (!(d < TC(1e-10))) {
                    gx += upr * dx; gy += upr * dy; gz += upr * dz;
                    lu += lt;
                    TC up = upr * d;
                    gsq += up * up;
                }
            }
            if (own) {
                for (int I = 0; I < NNUC; ++I) {
                    TC dx = xi - S.nuc[I][0], dy = yi - S.nuc[I][1], dz = zi - S.nuc[I][2];
                    TC d, ri;
                    dist(dx * dx + dy * dy + dz * dz, d, ri);
                    V -= S.Z[I] * ri;
                    TC uu, upr, lt;
                    pade_ab(S.enA[I], S.enB[I], d, ri, uu, upr, lt);
                    u -= uu;
                    if (!(d < TC(1e-10))) {
                        gx -= upr * dx; gy -= upr * dy; gz -= upr * dz;
                        lu -= lt;
                    }
                }
                TC ax = S.qa * gx, ay = S.qa * gy, az = S.qa * gz;
                TC lj = S.quirk_lap ? (lu + gsq) : (lu + gx * gx + gy * gy + gz * gz);
                TC lp = ld[sig] + 2 * (gdx[sig] * ax + gdy[sig] * ay + gdz[sig] * az) + lj;
                kin += lp;
                const int ecall = i;   // internal index; host permutes to caller order
                if (out_grad) {
                    out_grad[((size_t)w * NE + ecall) * 3 + 0] = (double)(gdx[sig] + ax);
                    out_grad[((size_t)w * NE + ecall) * 3 + 1] = (double)(gdy[sig] + ay);
                    out_grad[((size_t)w * NE + ecall) * 3 + 2] = (double)(gdz[sig] + az);
                }
                if (out_lap) out_lap[(size_t)w * NE + ecall] = (double)lp;
            }
        }
        u = wsum(u);
        V = wsum(V);
        kin = wsum(kin);
        if constexpr (std::is_same<TC, ff>::value)
            logdet = log((double)pmag) + (double)pexp * 0.6931471805599453;
        e_l = (double)(TC(-0.5) * kin + V + S.v_nn);
        if (lane == 0) {
            int fl = 0;
            if (!ok) fl |= FLAG_SINGULAR;
            if (!isfinite(e_l)) fl |= FLAG_NONFINITE;
            if (fl) atomicOr(flags, fl);
            if (write_state) { glog[w] = logdet + (double)u; gsign[w] = sg; gel[w] = e_l; }
        }
    }
    return act ? e_l : 0.0;
}

// Compensated sum of the block's per-warp values (lane 0 of each warp) into
// partial[2 slot], partial[2 slot + 1]; ends with a block barrier.
template <int WPB>
__device__ __forceinline__ void warp_block_partial(double v, double* partial, int slot) {
    __shared__ double ps[WPB];
    if ((threadIdx.x & 31) == 0) ps[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        Comp c{0.0, 0.0};
        for (int i = 0; i < WPB; ++i) c = comp_add(c, Comp{ps[i], 0.0});
        partial[2 * slot] = c.s;
        partial[2 * slot + 1] = c.c;
    }
    __syncthreads();
}

template <int NE, int NUP, int NNUC, class TC, class TS, int WPB>
__global__ void __launch_bounds__(32 * WPB) kw_measure(const SysW<TC>* __restrict__ Sg, const TS* __restrict__ gpos,
                                                       TS* __restrict__ gdinv, double* __restrict__ glog,
                                                       int* __restrict__ gsign, double* __restrict__ gel, int W,
                                                       int Wcap, int write_state, double* __restrict__ out_grad,
                                                       double* __restrict__ out_lap, double* partial, int* flags) {
    constexpr int NM = NUP > NE - NUP ? NUP : NE - NUP;
    __shared__ SysW<TC> S;
    extern __shared__ __align__(16) unsigned char wsm[];
    load_sysw(&S, Sg);
    const int wib = threadIdx.x >> 5;
    const int w = blockIdx.x * WPB + wib;
    TC* Mrow = reinterpret_cast<TC*>(wsm) + (size_t)wib * NM * MRS;   // [NM rows][MRS]
    double e_l = kw_measure_walker<NE, NUP, NNUC, TC, TS>(S, Mrow, gpos, gdinv, glog, gsign, gel, w, w < W, Wcap,
                                                          write_state, out_grad, out_lap, flags);
    if (partial) warp_block_partial<WPB>(e_l, partial, blockIdx.x);
}

// Batched form (compute type TC, state written, per-tile E_L partials), one
// block of WPB warps per WPB-walker tile.
template <int NE, int NUP, int NNUC, class TC, class TS, int WPB>
__global__ void __launch_bounds__(32 * WPB) kwb_measure(const BatchTile* __restrict__ tiles, int ntiles,
                                                        const BatchRec* __restrict__ recs, double* tile_partial) {
    constexpr int NM = NUP > NE - NUP ? NUP : NE - NUP;
    __shared__ SysW<TC> S;
    extern __shared__ __align__(16) unsigned char wsm[];
    if ((int)blockIdx.x >= ntiles) return;
    const int wib = threadIdx.x >> 5;
    TC* Mrow = reinterpret_cast<TC*>(wsm) + (size_t)wib * NM * MRS;
    const BatchTile tl = tiles[blockIdx.x];
    const BatchRec& R = recs[tl.rec];
    load_sysw(&S, static_cast<const SysW<TC>*>(R.tab_d));
    const int w = tl.w0 + wib;
    double e_l = kw_measure_walker<NE, NUP, NNUC, TC, TS>(S, Mrow, (const TS*)R.pos, (TS*)R.dinv, R.logabs, R.sign,
                                                          R.el, w, w < R.W, R.Wcap, 1, nullptr, nullptr, R.flags);
    warp_block_partial<WPB>(e_l, tile_partial, blockIdx.x);
}

int launch_sum_partials(const double* partial, int nblk, int nrows, double* out, cudaStream_t st);

// Per-shape launchers for the warp kernels.
template <int NE, int NUP, int NNUC>
struct WarpShapeOps {
    static constexpr int NM = NUP > NE - NUP ? NUP : NE - NUP;
    static constexpr int WPB = 4;
    // Batch tiles hold BTW walkers: BTW / WPB sweep blocks each, and one
    // refresh block of BTW warps (the wider refresh block shares the large
    // shared-memory table among more warps).
    static constexpr int BTW = 8;
    // dynamic shared memory of a sweep block: the WPB warps' proposal rows
    template <class T>
    static constexpr size_t sweep_smem() { return sizeof(T) * WPB * (size_t)sweep_scratch_elems<NE, NUP>(); }

    template <class T>
    static int table(const HostSys& hs, const SysW<T>** out) {
        // device copies of the table, cached per system and rebuilt when the
        // parameters or nuclei change (HostSys::version)
        const int slot = std::is_same<T, double>::value ? 0 : (std::is_same<T, float>::value ? 1 : 2);
        if (!hs.dev_table[slot] || hs.dev_table_version[slot] != hs.version) {
            SysW<T>* h = new SysW<T>;
            if (!fill_sysw<T>(hs, NE, NUP, NNUC, *h)) { delete h; return 7; }
            if (!hs.dev_table[slot]) {
                if (cudaMalloc(&hs.dev_table[slot], sizeof(SysW<T>)) != cudaSuccess) { delete h; return 8; }
            }
            cudaError_t e = cudaMemcpy(hs.dev_table[slot], h, sizeof(SysW<T>), cudaMemcpyHostToDevice);
            delete h;
            if (e != cudaSuccess) return 2;
            hs.dev_table_version[slot] = hs.version;
        }
        *out = static_cast<const SysW<T>*>(hs.dev_table[slot]);
        return 0;
    }

    static int init(const HostSys& hs, DevWalkers& dw, uint64_t seed, cudaStream_t st) {
        const SysW<double>* S;
        int rc = table<double>(hs, &S);
        if (rc) return rc;
        int n = NE * dw.W, tpb = 256;
        if (dw.prec == 0) kw_init<double><<<(n + tpb - 1) / tpb, tpb, 0, st>>>(S, (double*)dw.pos, NE, dw.W, dw.Wcap, seed);
        else kw_init<float><<<(n + tpb - 1) / tpb, tpb, 0, st>>>(S, (float*)dw.pos, NE, dw.W, dw.Wcap, seed);
        ++g_launch_count;
        return cudaGetLastError() == cudaSuccess ? 0 : 2;
    }

    template <class TC, class TS, int WB>
    static int measure_w(const HostSys& hs, DevWalkers& dw, bool ws, const MeasureOut& out, cudaStream_t st) {
        const SysW<TC>* S;
        int rc = table<TC>(hs, &S);
        if (rc) return rc;
        int nb = (dw.W + WB - 1) / WB;
        size_t smem = sizeof(TC) * WB * NM * MRS;
        auto kern = kw_measure<NE, NUP, NNUC, TC, TS, WB>;
        static bool attr = false;
        if (!attr) {
            if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
                return 2;
            attr = true;
        }
        double* partial = (ws && dw.partial && dw.partial_cap >= 2 * nb + 1) ? dw.partial : nullptr;
        kern<<<nb, 32 * WB, smem, st>>>(S, (const TS*)dw.pos, (TS*)dw.dinv, dw.logabs, dw.sign, dw.el, dw.W, dw.Wcap,
                                        ws ? 1 : 0, out.grad, out.lap, partial, dw.flags);
        ++g_launch_count;
        if (cudaGetLastError() != cudaSuccess) return 2;
        if (!partial) return 0;
        return launch_sum_partials(partial, nb, 1, dw.partial + dw.partial_cap - 1, st);
    }

    // Walkers per block of the standalone refresh, 4 or 8, chosen by timing.
    // The system table is per block and the row scratch per warp, so the two
    // shapes trade the table's fixed shared-memory cost against registers
    // per block; which keeps more warps resident and issues faster depends
    // on the arithmetic type.  A refresh recomputes the same state whatever
    // the block shape, so the first refresh of at least 1024 walkers per
    // arithmetic type (outside stream capture) runs both shapes, times each
    // once after a warm-up launch, and keeps the faster.
    static constexpr int WB_A = 4, WB_B = 8;

    template <class TC, class TS>
    static int measure2(const HostSys& hs, DevWalkers& dw, bool ws, const MeasureOut& out, cudaStream_t st) {
        static int best = 0;
        if (best == 0) {
            cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
            if (dw.W < 1024 || cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone)
                return measure_w<TC, TS, WB_A>(hs, dw, ws, out, st);
            cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
            int rc = 0;
            for (auto& e : ev)
                if (!rc && cudaEventCreate(&e) != cudaSuccess) rc = 2;
            if (!rc) rc = measure_w<TC, TS, WB_A>(hs, dw, ws, out, st);
            if (!rc) rc = measure_w<TC, TS, WB_B>(hs, dw, ws, out, st);
            if (!rc && cudaEventRecord(ev[0], st) != cudaSuccess) rc = 2;
            if (!rc) rc = measure_w<TC, TS, WB_A>(hs, dw, ws, out, st);
            if (!rc && cudaEventRecord(ev[1], st) != cudaSuccess) rc = 2;
            if (!rc) rc = measure_w<TC, TS, WB_B>(hs, dw, ws, out, st);
            if (!rc && cudaEventRecord(ev[2], st) != cudaSuccess) rc = 2;
            float ta = 0.0f, tb = 0.0f;
            if (!rc && cudaEventSynchronize(ev[2]) != cudaSuccess) rc = 2;
            if (!rc && (cudaEventElapsedTime(&ta, ev[0], ev[1]) != cudaSuccess ||
                        cudaEventElapsedTime(&tb, ev[1], ev[2]) != cudaSuccess))
                rc = 2;
            for (auto e : ev)
                if (e) cudaEventDestroy(e);
            if (!rc) best = tb < ta ? WB_B : WB_A;
            return rc;
        }
        return best == WB_B ? measure_w<TC, TS, WB_B>(hs, dw, ws, out, st)
                            : measure_w<TC, TS, WB_A>(hs, dw, ws, out, st);
    }

    static int measure(const HostSys& hs, DevWalkers& dw, int cp, bool ws, const MeasureOut& out, cudaStream_t st) {
        if (out.O || out.fhf || out.omega) return 7;
        // FP32 walkers refresh in float-float arithmetic on the FP32 pipe
        if (cp == 0) return dw.prec == 0 ? measure2<double, double>(hs, dw, ws, out, st)
                                         : measure2<ff, float>(hs, dw, ws, out, st);
        if (dw.prec == 1) return measure2<float, float>(hs, dw, ws, out, st);
        return 7;
    }

    template <class T, int MOVE>
    static int sweep_t(const HostSys& hs, DevWalkers& dw, int n, uint64_t s0, double step, double tau, double maxd,
                       uint64_t seed, cudaStream_t st) {
        const SysW<T>* S;
        int rc = table<T>(hs, &S);
        if (rc) return rc;
        int nb = (dw.W + WPB - 1) / WPB;
        auto kern = kw_sweep<NE, NUP, NNUC, T, MOVE, WPB>;
        const size_t smem = sweep_smem<T>();
        static bool attr = false;
        if (!attr) {
            if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
                return 2;
            attr = true;
        }
        kern<<<nb, 32 * WPB, smem, st>>>(S, (T*)dw.pos, (T*)dw.dinv, dw.sign, dw.W, dw.Wcap, n, s0, (T)step, (T)tau,
                                         (T)maxd, seed, dw.acc, dw.flags, dw.fixed_node);
        ++g_launch_count;
        return cudaGetLastError() == cudaSuccess ? 0 : 2;
    }

    // ---- batched launches ---------------------------------------------------
    // tab_s: the sweep table (walker precision); tab_d: the refresh table
    // (FP64 for FP64 walkers, float-float for FP32 walkers).
    static int batch_tables(const HostSys& hs, int prec, BatchRec& r) {
        r.ktab = nullptr;
        if (prec == 0) {
            const SysW<double>* d;
            int rc = table<double>(hs, &d);
            if (rc) return rc;
            r.tab_d = r.tab_s = d;
            return 0;
        }
        const SysW<ff>* m;
        const SysW<float>* f;
        int rc = table<ff>(hs, &m);
        if (!rc) rc = table<float>(hs, &f);
        if (rc) return rc;
        r.tab_d = m;
        r.tab_s = f;
        return 0;
    }

    template <class T, int MOVE>
    static int batch_sweep_t(const BatchClass& bc, const BatchCtl* ctl, cudaStream_t st, int* occ) {
        auto kern = kwb_sweep<NE, NUP, NNUC, T, MOVE, WPB, BTW>;
        const size_t smem = sweep_smem<T>();
        static bool attr = false;
        if (!attr) {
            if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
                return 2;
            attr = true;
        }
        if (occ) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, kern, 32 * WPB, smem) == cudaSuccess ? 0 : 2;
        if (bc.ntiles == 0) return 0;
        kern<<<bc.ntiles * (BTW / WPB), 32 * WPB, smem, st>>>(bc.tiles, bc.ntiles, bc.recs, ctl);
        ++g_launch_count;
        return cudaGetLastError() == cudaSuccess ? 0 : 2;
    }

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
        const size_t smem = sizeof(TC) * BTW * NM * MRS;
        auto kern = kwb_measure<NE, NUP, NNUC, TC, TS, BTW>;
        static bool attr = false;
        if (!attr) {
            if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
                return 2;
            attr = true;
        }
        if (occ) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, kern, 32 * BTW, smem) == cudaSuccess ? 0 : 2;
        if (bc.ntiles == 0) return 0;
        kern<<<bc.ntiles, 32 * BTW, smem, st>>>(bc.tiles, bc.ntiles, bc.recs, bc.tile_partial);
        ++g_launch_count;
        return cudaGetLastError() == cudaSuccess ? 0 : 2;
    }

    static int batch_measure(const BatchClass& bc, cudaStream_t st, int* occ = nullptr) {
        return bc.prec == 0 ? batch_measure_t<double, double>(bc, st, occ) : batch_measure_t<ff, float>(bc, st, occ);
    }

    static int sweep(const HostSys& hs, DevWalkers& dw, int mk, int n, uint64_t s0, double step, double tau,
                     double maxd, uint64_t seed, cudaStream_t st) {
        if (mk == MOVE_ONE_GAUSS)
            return dw.prec == 0 ? sweep_t<double, MOVE_ONE_GAUSS>(hs, dw, n, s0, step, tau, maxd, seed, st)
                                : sweep_t<float, MOVE_ONE_GAUSS>(hs, dw, n, s0, step, tau, maxd, seed, st);
        if (mk == MOVE_ONE_DRIFT)
            return dw.prec == 0 ? sweep_t<double, MOVE_ONE_DRIFT>(hs, dw, n, s0, step, tau, maxd, seed, st)
                                : sweep_t<float, MOVE_ONE_DRIFT>(hs, dw, n, s0, step, tau, maxd, seed, st);
        return 7;   // all-electron moves are not compiled for this shape
    }
};

}  // namespace qmc

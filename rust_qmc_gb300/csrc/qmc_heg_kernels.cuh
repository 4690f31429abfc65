// qmc_heg_kernels.cuh -- warp-per-walker kernels of the periodic homogeneous
// electron gas (src/systems/heg.rs): complex plane-wave determinants
// phi_k(r) = e^{i k.r}, a spin-dependent Jastrow with minimum image and a
// cutoff at L/2, and the Ewald Coulomb energy.
//
// Lane j holds column j of each complex inverse Slater matrix; lane k
// evaluates its own orbital e^{i k.r} (no AO contraction is needed).  The
// FP64 measurement rebuilds the inverses by complex Gauss-Jordan elimination
// and evaluates the Ewald sum: real-space pairs with images inside the erfc
// cutoff, reciprocal sum over a half-space k list (rho_k built from per-lane
// phase recursions and a warp reduction), and FP64 constants from the host.
#pragma once
#include <cstdio>
#include <cmath>
#include <cstring>
#include <vector>
#include "qmc_internal.h"
#include "qmc_device.cuh"

namespace qmc {

constexpr int HMAX_K = 1800;      // reciprocal half-space vectors (|n_i| <= 7 cube: 1687)

template <class T>
struct SysH {
    T L, invL, halfL;
    T F, pb, pc;                   // Jastrow: F, RPA b = 1/F, c = 0.2/F^2
    int form;                      // 0 Pade, 1 RPA, 2 Yukawa
    T a_ee[2];                     // [0] antiparallel, [1] parallel
    int quirk_cross;               // reference cross term without the orbital factor
    int real_images;               // 1: images inside the erfc cutoff; 0: minimum image only
    T alpha, rcut;
    double e_const;                // FP64 constant part of the Ewald energy
    double ksum_const;             // added per walker with the reciprocal sum
    T k2sum;                       // (1/2) sum over occupied |k|^2 of both sectors
    T kvec[2][32][3];              // [sector][column][xyz]
    int nk;
    int kmax;                      // reciprocal cutoff |n| <= kmax (sphere) or |n_i| <= kmax (cube)
    int kcube;                     // 1: the reference's full cube of integer vectors
    int perm[64];                  // internal -> caller electron index
};

// Reciprocal-space table of the Ewald sum (global memory, read uniformly).
struct KTable {
    int kint[HMAX_K][3];
    double kw[HMAX_K];
    float2 kwf[HMAX_K];            // kw as a float-float pair (hi, lo)
};

template <class T>
static bool fill_sysh(const HostSys& hs, int NE, int NUP, SysH<T>& S, KTable& KT) {
    std::memset(&S, 0, sizeof(S));
    std::memset(&KT, 0, sizeof(KT));
    for (int ei = 0; ei < hs.N && ei < 64; ++ei) S.perm[ei] = hs.perm[ei];
    if (hs.N != NE || hs.n_up != NUP || !(hs.box_L > 0)) return false;
    const double L = hs.box_L, V = L * L * L;
    S.L = (T)L; S.invL = (T)(1.0 / L); S.halfL = (T)(0.5 * L);
    S.F = (T)hs.F; S.pb = (T)(1.0 / hs.F); S.pc = (T)(0.2 / (hs.F * hs.F));
    S.form = (int)hs.jas[0];
    S.a_ee[0] = (T)hs.jas[2]; S.a_ee[1] = (T)hs.jas[3];
    S.quirk_cross = (hs.quirks & 8) ? 1 : 0;
    const bool qe = (hs.quirks & 4) != 0;
    const double alpha = qe ? 5.0 / L : hs.jas[4] / L;
    const int K = qe ? 7 : (int)hs.jas[5];
    S.alpha = (T)alpha;
    S.real_images = qe ? 0 : 1;
    S.rcut = (T)(5.6 / alpha);
    // the device sums the 27 nearest images: the cutoff must stay below 1.5 L
    if (!qe && 5.6 / alpha >= 1.5 * L) return false;
    // reciprocal half space; weight (4 pi / V) e^{-k^2 / 4 alpha^2} / k^2
    int nk = 0;
    double wsum = 0.0;
    const double dk = 2.0 * M_PI / L;
    for (int nx = 0; nx <= K; ++nx)
        for (int ny = -K; ny <= K; ++ny)
            for (int nz = -K; nz <= K; ++nz) {
                if (nx == 0 && (ny < 0 || (ny == 0 && nz <= 0))) continue;
                if (!qe && nx * nx + ny * ny + nz * nz > K * K) continue;
                if (nk >= HMAX_K) return false;
                double k2 = dk * dk * (nx * nx + ny * ny + nz * nz);
                KT.kint[nk][0] = nx; KT.kint[nk][1] = ny; KT.kint[nk][2] = nz;
                KT.kw[nk] = 4.0 * M_PI / V * std::exp(-k2 / (4.0 * alpha * alpha)) / k2;
                KT.kwf[nk].x = (float)KT.kw[nk];
                KT.kwf[nk].y = (float)(KT.kw[nk] - (double)KT.kwf[nk].x);
                wsum += KT.kw[nk];
                ++nk;
            }
    S.nk = nk;
    S.kmax = K;
    S.kcube = qe ? 1 : 0;
    const int N = hs.N;
    if (qe) {
        // heg.rs:526-581: (1/2) sum_k f_k (|rho_k|^2 - N) and -0.448 N / r_s
        const double rs = L / std::cbrt(4.0 * M_PI * N / 3.0);
        S.ksum_const = -N * wsum;
        S.e_const = -N * 0.448 / rs;
    } else {
        // one-component plasma: N [ (1/2) sum_{n!=0} erfc(alpha nL)/(nL) - alpha/sqrt(pi) - pi N/(2 V alpha^2) ]
        double img = 0.0;
        for (int a = -3; a <= 3; ++a)
            for (int b = -3; b <= 3; ++b)
                for (int c = -3; c <= 3; ++c) {
                    if (!a && !b && !c) continue;
                    double d = L * std::sqrt((double)(a * a + b * b + c * c));
                    img += std::erfc(alpha * d) / d;
                }
        S.ksum_const = 0.0;
        S.e_const = N * (0.5 * img - alpha / std::sqrt(M_PI) - M_PI * N / (2.0 * V * alpha * alpha));
    }
    double k2s = 0.0;
    for (int sig = 0; sig < 2; ++sig) {
        int col = 0;
        for (int ei = 0; ei < hs.N; ++ei) {
            int e = hs.perm[ei];
            if ((hs.spins[e] > 0) != (sig == 0)) continue;
            int k = hs.occ[e];
            if (col >= 32) return false;
            for (int c = 0; c < 3; ++c) S.kvec[sig][col][c] = (T)hs.kvec[3 * k + c];
            k2s += hs.kvec[3 * k] * hs.kvec[3 * k] + hs.kvec[3 * k + 1] * hs.kvec[3 * k + 1] +
                   hs.kvec[3 * k + 2] * hs.kvec[3 * k + 2];
            ++col;
        }
    }
    S.k2sum = (T)(0.5 * k2s);
    return true;
}

template <class T>
__device__ __forceinline__ void load_sysh(SysH<T>* dst, const SysH<T>* __restrict__ src, int bytes) {
    const int4* s = reinterpret_cast<const int4*>(src);
    int4* d = reinterpret_cast<int4*>(dst);
    const int n16 = bytes / (int)sizeof(int4);
    for (int i = threadIdx.x; i < n16; i += blockDim.x) d[i] = s[i];
    // tail words when the size is not a multiple of 16 bytes
    for (int i = n16 * 4 + threadIdx.x; i < bytes / 4; i += blockDim.x)
        reinterpret_cast<int*>(dst)[i] = reinterpret_cast<const int*>(src)[i];
    __syncthreads();
}

__device__ __forceinline__ void fsincos(double x, double* s, double* c) { sincos(x, s, c); }
__device__ __forceinline__ void fsincos(float x, float* s, float* c) { __sincosf(x, s, c); }
// float-float sine and cosine without FP64: Cody-Waite reduction
// r = x - n pi/2 with pi/2 in three FP32 parts (the leading difference is
// exact by Sterbenz's lemma, the n multiples by TwoProd), then the Taylor
// series on |r| <= pi/4 -- terms through r^7 (sine) and r^8 (cosine) in
// float-float, the rest (below 3.1e-7) in FP32 -- and the quadrant n mod 4.
// Absolute error below 1e-13 for |x| <= 60.
__device__ __forceinline__ void fsincos(ff x, ff* s, ff* c) {
    const float n = rintf(__fmul_rn(x.hi, 0.63661975f));
    const ff p = ff_two_prod(1.5707964f, n), q = ff_two_prod(-4.371139e-08f, n);
    ff r = ff(__fsub_rn(x.hi, p.hi)) + ff(x.lo);
    r = r + ff(-p.lo);
    r = r - q;
    r = r + ff(-__fmul_rn(-1.7151245e-15f, n));
    const ff r2 = r * r;
    const float h2 = r2.hi;
    // sin r = r + r^3 (-1/3! + r^2 (1/5! + r^2 (-1/7! + r^2 (1/9! - r^2/11! + r^4/13!))))
    const float qs = __fmul_rn(h2, __fmaf_rn(h2, __fmaf_rn(h2, 1.6059044e-10f, -2.5052108e-08f), 2.7557319e-06f));
    ff cs = ff(-1.0 / 5040.0) + ff(qs);
    cs = cs * r2 + ff(1.0 / 120.0);
    cs = cs * r2 + ff(-1.0 / 6.0);
    const ff sn = r + cs * r2 * r;
    // cos r = 1 + r^2 (-1/2 + r^2 (1/4! + r^2 (-1/6! + r^2 (1/8! + r^2 (-1/10! + r^2/12! - ...)))))
    const float qc = __fmaf_rn(h2, __fmaf_rn(h2, __fmaf_rn(h2, 4.7794773e-14f, -1.1470746e-11f), 2.0876757e-09f),
                               -2.7557319e-07f);
    ff cc = ff(1.0 / 40320.0) + ff(__fmul_rn(qc, h2));
    cc = cc * r2 + ff(-1.0 / 720.0);
    cc = cc * r2 + ff(1.0 / 24.0);
    cc = cc * r2 + ff(-0.5);
    const ff cn = ff(1.0f) + cc * r2;
    switch ((int)n & 3) {
        case 0: *s = sn; *c = cn; break;
        case 1: *s = cn; *c = -sn; break;
        case 2: *s = -sn; *c = -cn; break;
        default: *s = -cn; *c = sn; break;
    }
}

// erfc on [0, 6] in float-float arithmetic (0 beyond): the Chebyshev
// interpolant erfc(x) = c_0 / 2 + sum_{k=1..42} c_k T_k(t), t = x / 3 - 1,
// through 64 first-kind nodes (coefficients from gen_erfc_table.py, mpmath
// at 40 digits; |c_k| < 2e-18 beyond k = 42), summed by Clenshaw's
// recurrence: terms k >= 24 in FP32 (their partial sums stay below 1e-7),
// the rest in float-float.  Absolute error below 2e-14 on [0, 6].
static __constant__ const ff kErfcCheb[24] = {
    ff(3.673991e-01f, -6.9200334e-09f),
    ff(-3.3617035e-01f, 1.6510556e-09f),
    ff(2.5549158e-01f, 9.960313e-09f),
    ff(-1.5657288e-01f, 9.566121e-10f),
    ff(7.125926e-02f, -5.790789e-10f),
    ff(-1.7145663e-02f, 7.2621587e-10f),
    ff(-5.9834975e-03f, -6.355615e-11f),
    ff(9.309509e-03f, 1.6978224e-11f),
    ff(-5.190865e-03f, 1.0619118e-10f),
    ff(1.1763682e-03f, 4.8458522e-11f),
    ff(5.319446e-04f, 3.415539e-13f),
    ff(-6.203452e-04f, 1.8230945e-11f),
    ff(2.4648002e-04f, 1.3352023e-11f),
    ff(-4.3256662e-07f, -1.3714815e-14f),
    ff(-5.34781e-05f, 3.0843093e-13f),
    ff(2.795329e-05f, -6.6343177e-13f),
    ff(-3.1002157e-06f, 4.7403328e-14f),
    ff(-3.9868787e-06f, 1.6839862e-13f),
    ff(2.4134415e-06f, 3.8801173e-14f),
    ff(-3.3472375e-07f, 2.2182666e-15f),
    ff(-2.8443293e-07f, 9.959113e-15f),
    ff(1.730987e-07f, 5.6202656e-15f),
    ff(-2.0892596e-08f, -6.1127414e-16f),
    ff(-1.984897e-08f, -5.560824e-16f)};
static __constant__ const float kErfcChebTail[19] = {1.05052615e-08f, -7.149105e-10f, -1.2955014e-09f, 5.301936e-10f, 9.567597e-12f, -7.440549e-11f, 2.116448e-11f, 3.314318e-12f, -3.5774686e-12f, 5.862873e-13f, 2.661633e-13f, -1.3746954e-13f, 4.9925553e-15f, 1.3928812e-14f, -3.9142388e-15f, -5.4379457e-16f, 5.295314e-16f, -6.445588e-17f, -3.8180913e-17f};
__device__ __forceinline__ ff erfc_ff(ff x) {
    if (!(x.hi < 6.0f)) return ff(0.0f);
    const ff t = x * ff(1.0 / 3.0) - ff(1.0f);
    const float th2 = 2.0f * t.hi;
    float b1 = 0.0f, b2 = 0.0f;
#pragma unroll
    for (int k = 42; k >= 24; --k) {
        const float b0 = __fmaf_rn(th2, b1, __fsub_rn(kErfcChebTail[k - 24], b2));
        b2 = b1;
        b1 = b0;
    }
    ff B1 = ff(b1), B2 = ff(b2);
    const ff t2 = ff(2.0f * t.hi, 2.0f * t.lo);
#pragma unroll
    for (int k = 23; k >= 1; --k) {
        const ff B0 = t2 * B1 + kErfcCheb[k] - B2;
        B2 = B1;
        B1 = B0;
    }
    return ff(0.5f * kErfcCheb[0].hi, 0.5f * kErfcCheb[0].lo) + t * B1 - B2;
}

// Nearest integer of a float-float value (ties resolved by the leading part).
using ::rint;
__device__ __forceinline__ ff rint(ff x) {
    float r = rintf(x.hi);
    const float d = __fadd_rn(__fsub_rn(x.hi, r), x.lo);   // x.hi - r is exact
    if (d > 0.5f) r += 1.0f;
    else if (d < -0.5f) r -= 1.0f;
    return ff(r);
}

template <class T>
__device__ __forceinline__ T min_img(T d, const SysH<T>& S) { return d - S.L * rint(d * S.invL); }

// Warp shuffles for every compute type of the electron-gas kernels.
__device__ __forceinline__ float hshfl(float v, int s) { return __shfl_sync(0xffffffffu, v, s); }
__device__ __forceinline__ double hshfl(double v, int s) { return __shfl_sync(0xffffffffu, v, s); }
__device__ __forceinline__ ff hshfl(ff v, int s) { return wshfl(v, s); }

// |z|^2 of a pivot candidate on the leading parts (pivot choice only).
__device__ __forceinline__ float pivot_mag(float r, float i) { return r * r + i * i; }
__device__ __forceinline__ float pivot_mag(double r, double i) { return (float)(r * r + i * i); }
__device__ __forceinline__ float pivot_mag(ff r, ff i) { return r.hi * r.hi + i.hi * i.hi; }
__device__ __forceinline__ float hshfl_xor(float v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
__device__ __forceinline__ double hshfl_xor(double v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
__device__ __forceinline__ ff hshfl_xor(ff v, int m) { return shfl_xor(v, m); }

// Jastrow pair (src/systems/heg.rs:352-444): u, u'(r) and u'' + 2u'/r;
// zero outside (1e-10, L/2).
template <class T>
__device__ __forceinline__ void heg_u(const SysH<T>& S, T r, T a, T& u, T& du, T& lu) {
    u = 0; du = 0; lu = 0;
    if (!(r < S.halfL && r > T(1e-10))) return;
    if (S.form == 0) {
        T fr = S.F + r;
        u = a * r / (1 + r / S.F);
        du = a * S.F * S.F / (fr * fr);
        lu = 2 * a * S.F * S.F * S.F / (r * fr * fr * fr);
    } else if (S.form == 1) {
        T den = 1 + S.pb * r + S.pc * r * r;
        u = a * r / den;
        du = a * (1 - S.pc * r * r) / (den * den);
        T d2 = -a * 2 * (S.pc * r * den + (1 - S.pc * r * r) * (S.pb + 2 * S.pc * r)) / (den * den * den);
        lu = d2 + 2 / r * du;
    } else {
        T x = r / S.F, ex = fexp(-x), op = 1 + x;
        u = a * r * ex / op;
        du = a * ex * (1 - x - x * x) / (op * op);
        T d2 = a * ex / (S.F * S.F * op * op * op) * (-3 - 3 * x + x * x + x * x * x);
        lu = d2 + 2 / r * du;
    }
}

template <class T, int NE>
struct HLanePos {
    T x[2], y[2], z[2];
    __device__ __forceinline__ void get(int e, T& ex, T& ey, T& ez) const {
        T a = e < 32 ? x[0] : x[1], b = e < 32 ? y[0] : y[1], c = e < 32 ? z[0] : z[1];
        ex = hshfl(a, e & 31);
        ey = hshfl(b, e & 31);
        ez = hshfl(c, e & 31);
    }
    // Same, for an index that differs between lanes: the source lane cannot know which
    // half the reading lane wants, so both halves travel and the reader selects.
    __device__ __forceinline__ void get_own(int e, T& ex, T& ey, T& ez) const {
        const int s = e & 31;
        T x0 = hshfl(x[0], s), x1 = hshfl(x[1], s);
        T y0 = hshfl(y[0], s), y1 = hshfl(y[1], s);
        T z0 = hshfl(z[0], s), z1 = hshfl(z[1], s);
        ex = e < 32 ? x0 : x1; ey = e < 32 ? y0 : y1; ez = e < 32 ? z0 : z1;
    }
};

// Ewald weight of table entry t in the compute type.
template <class T>
__device__ __forceinline__ T kweight(const KTable* __restrict__ KT, int t) { return (T)KT->kw[t]; }
template <>
__device__ __forceinline__ ff kweight<ff>(const KTable* __restrict__ KT, int t) {
    const float2 w = KT->kwf[t];
    return ff(w.x, w.y);
}

template <class T>
__device__ __forceinline__ T hsum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += hshfl_xor(v, o);
    return v;
}

// u(r) alone, heg_u's expression for it, evaluated on every lane and masked
// (no divergent branch; out-of-range lanes may compute non-finite values).
template <class T>
__device__ __forceinline__ T heg_u_value(const SysH<T>& S, T r, T a) {
    T u;
    if (S.form == 0) {
        u = a * r / (1 + r / S.F);
    } else if (S.form == 1) {
        const T den = 1 + S.pb * r + S.pc * r * r;
        u = a * r / den;
    } else {
        const T x = r / S.F, ex = fexp(-x), op = 1 + x;
        u = a * r * ex / op;
    }
    return (r < S.halfL && r > T(1e-10)) ? u : T(0);
}

// Jastrow change (and gradients) for electron e moving o -> n.
template <int NE, int NUP, class T, bool GRAD>
__device__ __forceinline__ T hjastrow_delta(const SysH<T>& S, const HLanePos<T, NE>& P, int lane, int e, T ox, T oy,
                                            T oz, T nx, T ny, T nz, T (&go)[3], T (&gn)[3]) {
    T du = 0, g[6] = {0, 0, 0, 0, 0, 0};
    if constexpr (!GRAD) {
        // value only: every lane evaluates its partners and masks the unused ones
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            const int j = lane + 32 * r;
            const T a = S.a_ee[((j < NUP) == (e < NUP)) ? 1 : 0];
            T ax = min_img(ox - P.x[r], S), ay = min_img(oy - P.y[r], S), az = min_img(oz - P.z[r], S);
            T bx = min_img(nx - P.x[r], S), by = min_img(ny - P.y[r], S), bz = min_img(nz - P.z[r], S);
            T ra = fsqrt(ax * ax + ay * ay + az * az), rb = fsqrt(bx * bx + by * by + bz * bz);
            const T d = heg_u_value(S, rb, a) - heg_u_value(S, ra, a);
            du += (j < NE && j != e) ? d : T(0);
        }
        return hsum(du);
    } else {
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            const int j = lane + 32 * r;
            if (j < NE && j != e) {
                const T a = S.a_ee[((j < NUP) == (e < NUP)) ? 1 : 0];
                T ax = min_img(ox - P.x[r], S), ay = min_img(oy - P.y[r], S), az = min_img(oz - P.z[r], S);
                T bx = min_img(nx - P.x[r], S), by = min_img(ny - P.y[r], S), bz = min_img(nz - P.z[r], S);
                T ra = fsqrt(ax * ax + ay * ay + az * az), rb = fsqrt(bx * bx + by * by + bz * bz);
                T ua, dua, lua, ub, dub, lub;
                heg_u(S, ra, a, ua, dua, lua);
                heg_u(S, rb, a, ub, dub, lub);
                du += ub - ua;
                if (GRAD) {
                    T fa = ra > 0 ? dua / ra : T(0), fb = rb > 0 ? dub / rb : T(0);
                    g[0] += fa * ax; g[1] += fa * ay; g[2] += fa * az;
                    g[3] += fb * bx; g[4] += fb * by; g[5] += fb * bz;
                }
            }
        }
        du = hsum(du);
        if (GRAD) {
            go[0] = hsum(g[0]); go[1] = hsum(g[1]); go[2] = hsum(g[2]);
            gn[0] = hsum(g[3]); gn[1] = hsum(g[4]); gn[2] = hsum(g[5]);
        }
        return du;
    }
}

template <class TS>
__global__ void khw_init(const SysH<double>* __restrict__ S, TS* __restrict__ pos, int NE, int W, int Wcap,
                         uint64_t seed) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= NE * W) return;
    int e = i / W, w = i - e * W;
    U4 x = rng_draw(seed, (uint32_t)w, 0, (uint32_t)S->perm[e], TAG_INIT);
    double L = S->L;
    pos[(3 * e + 0) * (size_t)Wcap + w] = (TS)(L * to_u01(x.x, 0.0));
    pos[(3 * e + 1) * (size_t)Wcap + w] = (TS)(L * to_u01(x.y, 0.0));
    pos[(3 * e + 2) * (size_t)Wcap + w] = (TS)(L * to_u01(x.z, 0.0));
}

// Single-electron sweeps, one warp per walker.
template <class T> struct HComplex;
template <> struct HComplex<float> { using type = float2; };
template <> struct HComplex<double> { using type = double2; };
// Shared bytes per warp of the sweep's inverse columns (both sectors).
template <int NM, class T>
__host__ __device__ constexpr size_t hsweep_warp_bytes() { return sizeof(T) * 2 * 2 * NM * 32; }

// A is const volatile SweepArgs<T> (block-shared; see SweepArgs).
template <int NE, int NUP, class T, int MOVE, class A>
__device__ __forceinline__ void khw_sweep_walker(const SysH<T>& S, A& a, typename HComplex<T>::type* Dsh, int w) {
    constexpr int NDN = NE - NUP;
    constexpr int NM = NUP > NDN ? NUP : NDN;
    const int lane = threadIdx.x & 31;
    HLanePos<T, NE> P;
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        const int j = lane + 32 * r;
        const bool ok = j < NE;
        P.x[r] = ok ? a.pos[(3 * j + 0) * (size_t)a.Wcap + w] : T(0);
        P.y[r] = ok ? a.pos[(3 * j + 1) * (size_t)a.Wcap + w] : T(0);
        P.z[r] = ok ? a.pos[(3 * j + 2) * (size_t)a.Wcap + w] : T(0);
    }
    // complex inverse columns in the warp's shared rows: Dsh[(sig NM + k) 32 + lane]
    // = D^-1[k][lane] (re, im) of sector sig; each lane touches only its own
    // column (HBM storage [2][NM*NM][2][Wcap])
    using C2 = typename HComplex<T>::type;
#pragma unroll
    for (int k = 0; k < NM; ++k) {
        size_t b0 = ((size_t)(0 * NM * NM + k * NM + lane)) * 2 * a.Wcap, b1 = ((size_t)(1 * NM * NM + k * NM + lane)) * 2 * a.Wcap;
        C2 d0, d1;
        d0.x = lane < NUP ? a.dinv[b0 + w] : T(0);
        d0.y = lane < NUP ? a.dinv[b0 + a.Wcap + w] : T(0);
        d1.x = lane < NDN ? a.dinv[b1 + w] : T(0);
        d1.y = lane < NDN ? a.dinv[b1 + a.Wcap + w] : T(0);
        Dsh[(0 * NM + k) * 32 + lane] = d0;
        Dsh[(1 * NM + k) * 32 + lane] = d1;
    }
    unsigned acc = 0;
    int flg = 0;
    for (int it = 0; it < a.n_sweeps; ++it) {
        const uint64_t st = a.step0 + (uint64_t)it;
#pragma unroll
        for (int sig = 0; sig < 2; ++sig) {
            C2* Dc = Dsh + sig * NM * 32 + lane;      // Dc[k * 32] = D^-1[k][lane]
            const int NS = sig == 0 ? NUP : NDN;
            const T kx = S.kvec[sig][lane][0], ky = S.kvec[sig][lane][1], kz = S.kvec[sig][lane][2];
            static_assert(NUP <= 32 && NE - NUP <= 32, "one lane per sector electron");
            const MoveDraw<T> draws = sector_draws<T>(a.seed, (uint32_t)w, st, sig * NUP, NS, lane);
            T csr = 1, csi = 0;                        // pending complex scale of this lane's column (Gaussian moves)
            for (int q = 0; q < NS; ++q) {
                const int e = sig * NUP + q;
                T rx, ry, rz;
                P.get(e, rx, ry, rz);
                const MoveDraw<T> md = draw_of(draws, q);
                T nx, ny, nz, logG = 0, dlx = 0, dly = 0, dlz = 0;
                if (MOVE == MOVE_ONE_DRIFT) {
                    // Re(grad ln D) at the current position: lane l sums (i k_j phi_j) Dinv[j][l]
                    T s, c;
                    fsincos(kx * rx + ky * ry + kz * rz, &s, &c);
                    T ax = 0, ay = 0, az = 0;
#pragma unroll 9
                    for (int j = 0; j < NM; ++j) {
                        T pr = __shfl_sync(0xffffffffu, c, j), pi = __shfl_sync(0xffffffffu, s, j);
                        T kjx = S.kvec[sig][j][0], kjy = S.kvec[sig][j][1], kjz = S.kvec[sig][j][2];
                        // Re(i k phi D) = -k Im(phi D)
                        const C2 d = Dc[j * 32];
                        T im = pr * d.y + pi * d.x;
                        ax -= kjx * im; ay -= kjy * im; az -= kjz * im;
                    }
                    ax = __shfl_sync(0xffffffffu, ax, q); ay = __shfl_sync(0xffffffffu, ay, q); az = __shfl_sync(0xffffffffu, az, q);
                    T g0[3], g1[3];
                    hjastrow_delta<NE, NUP, T, true>(S, P, lane, e, rx, ry, rz, rx, ry, rz, g0, g1);
                    const T tau = a.tau, maxd = a.maxd;
                    dlx = tau * 2 * (ax + g0[0]); dly = tau * 2 * (ay + g0[1]); dlz = tau * 2 * (az + g0[2]);
                    T m = fsqrt(dlx * dlx + dly * dly + dlz * dlz);
                    if (m > maxd) { T sc = maxd / m; dlx *= sc; dly *= sc; dlz *= sc; }
                    T sd2 = fsqrt(2 * tau);
                    nx = rx + dlx + sd2 * md.n0; ny = ry + dly + sd2 * md.n1; nz = rz + dlz + sd2 * md.n2;
                } else {
                    const T step = a.step;
                    nx = rx + step * md.n0; ny = ry + step * md.n1; nz = rz + step * md.n2;
                }
                T ps, pc;
                fsincos(kx * nx + ky * ny + kz * nz, &ps, &pc);
                // t_l = sum_j phi_j Dinv[j][l]; R = t_q
                T tr = 0, ti = 0;
#pragma unroll 9
                for (int j = 0; j < NM; ++j) {
                    T pr = __shfl_sync(0xffffffffu, pc, j), pi = __shfl_sync(0xffffffffu, ps, j);
                    const C2 d = Dc[j * 32];
                    tr += pr * d.x - pi * d.y;
                    ti += pr * d.y + pi * d.x;
                }
                const T Rr = __shfl_sync(0xffffffffu, tr, q), Ri = __shfl_sync(0xffffffffu, ti, q);
                const T R2 = Rr * Rr + Ri * Ri;
                T g0[3], gn[3];
                T du = hjastrow_delta<NE, NUP, T, MOVE == MOVE_ONE_DRIFT>(S, P, lane, e, rx, ry, rz, nx, ny, nz, g0, gn);
                if (MOVE == MOVE_ONE_DRIFT) {
                    // Re(grad ln D') = Re(G / R) with G = sum_j i k_j phi_j(r') Dinv[j][q]
                    T Gx_r = 0, Gy_r = 0, Gz_r = 0, Gx_i = 0, Gy_i = 0, Gz_i = 0;
#pragma unroll 9
                    for (int j = 0; j < NM; ++j) {
                        T pr = __shfl_sync(0xffffffffu, pc, j), pi = __shfl_sync(0xffffffffu, ps, j);
                        const C2 d = Dc[j * 32];
                        T re = pr * d.x - pi * d.y, im = pr * d.y + pi * d.x;
                        T kjx = S.kvec[sig][j][0], kjy = S.kvec[sig][j][1], kjz = S.kvec[sig][j][2];
                        Gx_r -= kjx * im; Gy_r -= kjy * im; Gz_r -= kjz * im;
                        Gx_i += kjx * re; Gy_i += kjy * re; Gz_i += kjz * re;
                    }
                    Gx_r = __shfl_sync(0xffffffffu, Gx_r, q); Gy_r = __shfl_sync(0xffffffffu, Gy_r, q); Gz_r = __shfl_sync(0xffffffffu, Gz_r, q);
                    Gx_i = __shfl_sync(0xffffffffu, Gx_i, q); Gy_i = __shfl_sync(0xffffffffu, Gy_i, q); Gz_i = __shfl_sync(0xffffffffu, Gz_i, q);
                    const T tau = a.tau, maxd = a.maxd;
                    T iR2 = R2 > 0 ? T(1) / R2 : T(0);
                    // Re(G / R) = (G_r R_r + G_i R_i) / |R|^2
                    T cx = (Gx_r * Rr + Gx_i * Ri) * iR2 + gn[0];
                    T cy = (Gy_r * Rr + Gy_i * Ri) * iR2 + gn[1];
                    T cz = (Gz_r * Rr + Gz_i * Ri) * iR2 + gn[2];
                    cx *= 2 * tau; cy *= 2 * tau; cz *= 2 * tau;
                    T m = fsqrt(cx * cx + cy * cy + cz * cz);
                    if (m > maxd) { T sc = maxd / m; cx *= sc; cy *= sc; cz *= sc; }
                    T fx = nx - rx - dlx, fy = ny - ry - dly, fz = nz - rz - dlz;
                    T qx = rx - nx - cx, qy = ry - ny - cy, qz = rz - nz - cz;
                    logG = ((fx * fx + fy * fy + fz * fz) - (qx * qx + qy * qy + qz * qz)) / (4 * tau);
                }
                T prob = R2 * fexp(2 * du);
                if (MOVE == MOVE_ONE_DRIFT) prob *= fexp(logG);
                if (prob != prob) flg |= FLAG_NONFINITE;
                if (md.uacc < prob && R2 > T(0)) {
                    // wrap the new position into the box
                    T wx = nx - S.L * floor(nx * S.invL), wy = ny - S.L * floor(ny * S.invL), wz = nz - S.L * floor(nz * S.invL);
                    if ((e & 31) == lane) {
                        if (e < 32) { P.x[0] = wx; P.y[0] = wy; P.z[0] = wz; }
                        else { P.x[1] = wx; P.y[1] = wy; P.z[1] = wz; }
                    }
                    // complex Sherman-Morrison: D'[k][l] = D[k][l] - D[k][q] t_l / R, D'[k][q] = D[k][q] / R
                    const T iR2 = T(1) / R2;
                    const T iRr = Rr * iR2, iRi = -Ri * iR2;              // 1/R
                    T fr = tr * iRr - ti * iRi, fi = tr * iRi + ti * iRr;   // t_l / R
                    if constexpr (MOVE == MOVE_ONE_GAUSS) {
                        // column q keeps its values and takes the factor 1/R when the
                        // sector ends (a column's scale is 1 until its own electron
                        // moves, so t_q and R are read unscaled)
                        if (lane == q) { fr = 0; fi = 0; csr = iRr; csi = iRi; }
#pragma unroll 9
                        for (int k = 0; k < NM; ++k) {
                            const C2 d = Dc[k * 32];
                            T qr = __shfl_sync(0xffffffffu, d.x, q), qi = __shfl_sync(0xffffffffu, d.y, q);
                            C2 n;
                            n.x = d.x - (qr * fr - qi * fi); n.y = d.y - (qr * fi + qi * fr);
                            Dc[k * 32] = n;
                        }
                    } else {
#pragma unroll 9
                        for (int k = 0; k < NM; ++k) {
                            const C2 d = Dc[k * 32];
                            T qr = __shfl_sync(0xffffffffu, d.x, q), qi = __shfl_sync(0xffffffffu, d.y, q);
                            C2 n;
                            if (lane == q) { n.x = qr * iRr - qi * iRi; n.y = qr * iRi + qi * iRr; }
                            else { n.x = d.x - (qr * fr - qi * fi); n.y = d.y - (qr * fi + qi * fr); }
                            Dc[k * 32] = n;
                        }
                    }
                    ++acc;
                }
            }
            if constexpr (MOVE == MOVE_ONE_GAUSS) {
#pragma unroll 9
                for (int k = 0; k < NM; ++k) {
                    const C2 d = Dc[k * 32];
                    C2 n;
                    n.x = d.x * csr - d.y * csi; n.y = d.x * csi + d.y * csr;
                    Dc[k * 32] = n;
                }
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
        size_t b0 = ((size_t)(0 * NM * NM + k * NM + lane)) * 2 * a.Wcap, b1 = ((size_t)(1 * NM * NM + k * NM + lane)) * 2 * a.Wcap;
        const C2 d0 = Dsh[(0 * NM + k) * 32 + lane], d1 = Dsh[(1 * NM + k) * 32 + lane];
        if (lane < NUP) { a.dinv[b0 + w] = d0.x; a.dinv[b0 + a.Wcap + w] = d0.y; }
        if (lane < NDN) { a.dinv[b1 + w] = d1.x; a.dinv[b1 + a.Wcap + w] = d1.y; }
    }
    if (lane == 0) {
        if (acc) atomicAdd(a.acc, (unsigned long long)acc);
        if (flg) atomicOr(a.flags, flg);
    }
}

template <int NE, int NUP, class T, int MOVE, int WPB>
// 16 warps per SM for FP32 walkers (four blocks of four: 56 KB of shared
// memory each, at most 128 registers), 8 for FP64 walkers.
__global__ void __launch_bounds__(32 * WPB, (sizeof(T) == 4 ? 16 : 8) / WPB) khw_sweep(const SysH<T>* __restrict__ Sg, T* __restrict__ gpos,
                                                      T* __restrict__ gdinv, int W, int Wcap, int n_sweeps,
                                                      uint64_t step0, T step, T tau, T maxd, uint64_t seed,
                                                      unsigned long long* acc_out, int* flags) {
    constexpr int NM = NUP > NE - NUP ? NUP : NE - NUP;
    __shared__ SysH<T> S;
    __shared__ SweepArgs<T> args;
    extern __shared__ __align__(16) unsigned char hsm[];
    if (threadIdx.x == 0)
        args = SweepArgs<T>{gpos, gdinv, nullptr, acc_out, flags, step0, seed, step, tau, maxd, W, Wcap, n_sweeps, 0};
    load_sysh(&S, Sg, (int)sizeof(SysH<T>));   // ends with a block barrier
    const int w = blockIdx.x * WPB + (threadIdx.x >> 5);
    if (w >= W) return;
    auto* Dsh = reinterpret_cast<typename HComplex<T>::type*>(hsm) + (size_t)(threadIdx.x >> 5) * 2 * NM * 32;
    const volatile SweepArgs<T>& a = args;
    khw_sweep_walker<NE, NUP, T, MOVE>(S, a, Dsh, w);
}

// Batched form: one block per (system, WPB-walker tile); the hardware block
// scheduler balances uneven systems and classes that run side by side.
template <int NE, int NUP, class T, int MOVE, int WPB>
__global__ void __launch_bounds__(32 * WPB, (sizeof(T) == 4 ? 16 : 8) / WPB) khwb_sweep(const BatchTile* __restrict__ tiles, int ntiles,
                                                       const BatchRec* __restrict__ recs,
                                                       const BatchCtl* __restrict__ ctl) {
    constexpr int NM = NUP > NE - NUP ? NUP : NE - NUP;
    __shared__ SysH<T> S;
    __shared__ SweepArgs<T> args;
    extern __shared__ __align__(16) unsigned char hsm[];
    if ((int)blockIdx.x >= ntiles) return;
    auto* Dsh = reinterpret_cast<typename HComplex<T>::type*>(hsm) + (size_t)(threadIdx.x >> 5) * 2 * NM * 32;
    const BatchTile tl = tiles[blockIdx.x];
    if (threadIdx.x == 0) args = sweep_args<T>(recs[tl.rec], *ctl);
    load_sysh(&S, static_cast<const SysH<T>*>(recs[tl.rec].tab_s), (int)sizeof(SysH<T>));   // ends with a barrier
    const volatile SweepArgs<T>& a = args;
    const int w = tl.w0 + (int)(threadIdx.x >> 5);
    if (w >= a.W) return;
    khw_sweep_walker<NE, NUP, T, MOVE>(S, a, Dsh, w);
}

// FP64 (or FP32) full evaluation: complex Gauss-Jordan, kinetic terms, Ewald.
// PART 0: the whole refresh.  The float-float refresh of FP32 walkers can
// also run as two launches over per-walker scratch drows [7][NE][Wcap]:
// PART 1, the determinant half (orbital matrix, inverse, log|D| into glog,
// grad ln D and lap D / D per electron into drows), and PART 2, the energy
// half (Jastrow, Ewald sums, E_L), which reads them back.  Each launch
// carries half the code and PART 2 none of the inversion's registers.
template <int NE, int NUP, class TC, class TS, int PART, class A>
__device__ __forceinline__ double khw_measure_walker(const SysH<TC>& S, A& a, TC* Mr, int w, bool act) {
    static_assert(PART == 0 || std::is_same<TC, ff>::value, "the two-part refresh is float-float only");
    constexpr int NDN = NE - NUP;
    constexpr int NM = NUP > NDN ? NUP : NDN;
    const int lane = threadIdx.x & 31;
    TC* Mi = Mr + NM * 32;                            // Mr: [re|im][row][lane]
    double e_l = 0.0;
    if (act) {
        HLanePos<TC, NE> P;
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            const int j = lane + 32 * r;
            const bool ok = j < NE;
            P.x[r] = ok ? (TC)a.pos[(3 * j + 0) * (size_t)a.Wcap + w] : TC(0);
            P.y[r] = ok ? (TC)a.pos[(3 * j + 1) * (size_t)a.Wcap + w] : TC(0);
            P.z[r] = ok ? (TC)a.pos[(3 * j + 2) * (size_t)a.Wcap + w] : TC(0);
        }
        double logdet = 0.0;
        ff pmag = ff(1.0f);                       // float-float form: |det|^2 = pmag 2^pexp
        int pexp = 0;
        bool ok = true;
        TC gdx[2] = {0, 0}, gdy[2] = {0, 0}, gdz[2] = {0, 0}, gqx[2] = {0, 0}, gqy[2] = {0, 0}, gqz[2] = {0, 0};
        TC ldet[2] = {0, 0};
        if constexpr (PART != 2) {
#pragma unroll
        for (int sig = 0; sig < 2; ++sig) {
            const int NS = sig == 0 ? NUP : NDN;
            const TC kx = S.kvec[sig][lane][0], ky = S.kvec[sig][lane][1], kz = S.kvec[sig][lane][2];
            for (int q = 0; q < NS; ++q) {
                TC rx, ry, rz;
                P.get(sig * NUP + q, rx, ry, rz);
                TC s, c;
                fsincos(kx * rx + ky * ry + kz * rz, &s, &c);
                Mr[q * 32 + lane] = c;
                Mi[q * 32 + lane] = s;
            }
            __syncwarp();
            // complex Gauss-Jordan in place: lane j carries column j of D and
            // ends with column j of D^-1.  Step k: pivot row p by |D[i][k]|,
            // rows k and p interchanged; with a = D[k][k], row k is divided by
            // a, column k becomes -D[i][k]/a (and 1/a on the diagonal), the rest
            // loses D[i][k] x row k.  Lane k's own update is the same form with
            // t = 1 + 1/a.  The row interchanges are undone at the end as column
            // interchanges in reverse order: lane j gathers column src(j),
            // src = tau_{n-1}( ... tau_0(j)), tau_k the swap of k and p_k.
            // The pivot loop is rolled (one copy of the step's code, which an
            // unrolled loop would repeat NS times): the registers hold the rows
            // rotated so that row k sits in register 0 at step k -- the rows not
            // yet pivoted in registers 0..NS-1-k, in the unrolled form's order,
            // the pivoted ones after them -- and each step ends by moving
            // register 0 to the back.  After NS steps the order is row k in
            // register k again.
            TC Ar[NM], Ai[NM];
#pragma unroll
            for (int i = 0; i < NM; ++i) {
                bool in = i < NS && lane < NS;
                Ar[i] = in ? Mr[i * 32 + lane] : TC(i == lane ? 1 : 0);
                Ai[i] = in ? Mi[i * 32 + lane] : TC(0);
            }
            int src = lane;
#pragma unroll 1
            for (int k = 0; k < NS; ++k) {
                // pivot: the largest |D[i][k]| over the rows not yet pivoted
                // (leading parts; the first of equal ones)
                int p = 0;
                float best = pivot_mag(Ar[0], Ai[0]);
#pragma unroll
                for (int r = 1; r < NM; ++r) {
                    const float m = pivot_mag(Ar[r], Ai[r]);
                    if (r < NS - k && m > best) { best = m; p = r; }
                }
                p = __shfl_sync(0xffffffffu, p, k);
#pragma unroll
                for (int r = 1; r < NM; ++r) {
                    const bool sw = (r == p);
                    TC a = Ar[0], b = Ar[r]; Ar[0] = sw ? b : a; Ar[r] = sw ? a : b;
                    a = Ai[0]; b = Ai[r]; Ai[0] = sw ? b : a; Ai[r] = sw ? a : b;
                }
                const int pk = k + p;
                src = (src == k) ? pk : ((src == pk) ? k : src);
                TC pr = hshfl(Ar[0], k), pi = hshfl(Ai[0], k);
                TC pa = pr * pr + pi * pi;
                if (!(pa > TC(0))) { ok = false; pr = 1; pi = 0; pa = 1; }
                if constexpr (std::is_same<TC, ff>::value) {
                    pmag = pmag * pa;                  // |det|^2 as a rescaled product
                    ff_rescale(pmag, pexp);
                } else {
                    logdet += 0.5 * log((double)pa);
                }
                const TC ipr = pr / pa, ipi = -pi / pa;           // 1/a
                TC tr, ti;
                if (lane == k) {
                    tr = TC(1) + ipr; ti = ipi;
                    Ar[0] = ipr; Ai[0] = ipi;
                } else {
                    tr = Ar[0] * ipr - Ai[0] * ipi; ti = Ar[0] * ipi + Ai[0] * ipr;
                    Ar[0] = tr; Ai[0] = ti;
                }
#pragma unroll
                for (int i = 1; i < NM; ++i) {
                    if (i >= NS) continue;
                    TC fr = hshfl(Ar[i], k), fi = hshfl(Ai[i], k);
                    Ar[i] -= fr * tr - fi * ti; Ai[i] -= fr * ti + fi * tr;
                }
                // rotate registers 0..NS-1 by one: the pivoted row goes last
                const TC r0 = Ar[0], i0 = Ai[0];
#pragma unroll
                for (int i = 0; i + 1 < NM; ++i) {
                    if (i + 1 < NS) { Ar[i] = Ar[i + 1]; Ai[i] = Ai[i + 1]; }
                    else if (i + 1 == NS) { Ar[i] = r0; Ai[i] = i0; }
                }
                if (NS == NM) { Ar[NM - 1] = r0; Ai[NM - 1] = i0; }
            }
            // unscramble: lane j takes column src(j)
#pragma unroll
            for (int i = 0; i < NM; ++i) {
                if (i >= NS) break;
                Ar[i] = hshfl(Ar[i], src);
                Ai[i] = hshfl(Ai[i], src);
            }
            TC (&Ir)[NM] = Ar;
            TC (&Ii)[NM] = Ai;
            if (a.write_state && lane < NS) {
#pragma unroll
                for (int k = 0; k < NM; ++k) {
                    if (k >= NS) break;
                    size_t b = ((size_t)(sig * NM * NM + k * NM + lane)) * 2 * a.Wcap;
                    a.dinv[b + w] = (TS)Ir[k];
                    a.dinv[b + a.Wcap + w] = (TS)Ii[k];
                }
            }
            // lane = electron row q: grad ln D = sum_j Dinv[j][q] i k_j phi_j(r_q); lap D / D = -sum_j Dinv phi k^2
            if (lane < NS) {
                TC ax = 0, ay = 0, az = 0, bx = 0, by = 0, bz = 0, lr = 0;
#pragma unroll
                for (int j = 0; j < NM; ++j) {
                    if (j >= NS) break;
                    TC pr = Mr[lane * 32 + j], pi = Mi[lane * 32 + j];
                    TC re = pr * Ir[j] - pi * Ii[j], im = pr * Ii[j] + pi * Ir[j];
                    TC kjx = S.kvec[sig][j][0], kjy = S.kvec[sig][j][1], kjz = S.kvec[sig][j][2];
                    ax -= kjx * im; ay -= kjy * im; az -= kjz * im;                 // Re(i k w phi)
                    bx -= kjx * Ii[j]; by -= kjy * Ii[j]; bz -= kjz * Ii[j];         // Re(i k w), reference form
                    lr -= (kjx * kjx + kjy * kjy + kjz * kjz) * re;
                }
                gdx[sig] = ax; gdy[sig] = ay; gdz[sig] = az;
                gqx[sig] = bx; gqy[sig] = by; gqz[sig] = bz;
                ldet[sig] = lr;
            }
            __syncwarp();
        }
        if constexpr (std::is_same<TC, ff>::value)
            logdet = 0.5 * (log((double)pmag) + (double)pexp * 0.6931471805599453);
        }
        if constexpr (PART == 1) {
#pragma unroll
            for (int sig = 0; sig < 2; ++sig) {
                const int NS = sig == 0 ? NUP : NDN;
                if (lane < NS) {
                    const int i = sig * NUP + lane;
                    const TC v[7] = {gdx[sig], gdy[sig], gdz[sig], gqx[sig], gqy[sig], gqz[sig], ldet[sig]};
#pragma unroll
                    for (int c = 0; c < 7; ++c) ff_store(a.rows + (size_t)(c * NE + i) * a.Wcap + w, v[c]);
                }
            }
            if (lane == 0) {
                if (!ok) atomicOr(a.flags, FLAG_SINGULAR);
                a.log[w] = logdet;
            }
            return 0.0;
        }
        if constexpr (PART == 2) {
#pragma unroll
            for (int sig = 0; sig < 2; ++sig) {
                const int NS = sig == 0 ? NUP : NDN;
                if (lane < NS) {
                    const int i = sig * NUP + lane;
                    TC v[7];
#pragma unroll
                    for (int c = 0; c < 7; ++c) v[c] = ff_load(a.rows + (size_t)(c * NE + i) * a.Wcap + w);
                    gdx[sig] = v[0]; gdy[sig] = v[1]; gdz[sig] = v[2];
                    gqx[sig] = v[3]; gqy[sig] = v[4]; gqz[sig] = v[5]; ldet[sig] = v[6];
                }
            }
            logdet = a.log[w];
        }
        // Jastrow for this lane's electrons (pairs from both ends)
        TC u = 0, kin = 0;
#pragma unroll
        for (int sig = 0; sig < 2; ++sig) {
            const int NS = sig == 0 ? NUP : NDN;
            const int i = sig * NUP + lane;
            const bool own = lane < NS;
            TC xi, yi, zi;
            P.get_own(min(i, NE - 1), xi, yi, zi);
            TC gx = 0, gy = 0, gz = 0, lu = 0;
            for (int j = 0; j < NE; ++j) {
                TC xj, yj, zj;
                P.get(j, xj, yj, zj);
                if (!own || j == i) continue;
                const TC a = S.a_ee[((j < NUP) == (i < NUP)) ? 1 : 0];
                TC dx = min_img(xi - xj, S), dy = min_img(yi - yj, S), dz = min_img(zi - zj, S);
                TC r = fsqrt(dx * dx + dy * dy + dz * dz);
                TC uu, du, l;
                heg_u(S, r, a, uu, du, l);
                u += TC(0.5) * uu;
                if (r < S.halfL && r > TC(1e-10)) {
                    TC f = du / r;
                    gx += f * dx; gy += f * dy; gz += f * dz;
                    lu += l;
                }
            }
            if (own) {
                TC cx = S.quirk_cross ? gqx[sig] : gdx[sig], cy = S.quirk_cross ? gqy[sig] : gdy[sig],
                   cz = S.quirk_cross ? gqz[sig] : gdz[sig];
                TC lp = ldet[sig] + lu + gx * gx + gy * gy + gz * gz + 2 * (cx * gx + cy * gy + cz * gz);
                kin += lp;
                if (a.grad) {
                    a.grad[((size_t)w * NE + i) * 3 + 0] = (double)(gdx[sig] + gx);
                    a.grad[((size_t)w * NE + i) * 3 + 1] = (double)(gdy[sig] + gy);
                    a.grad[((size_t)w * NE + i) * 3 + 2] = (double)(gdz[sig] + gz);
                }
                if (a.lap) a.lap[(size_t)w * NE + i] = (double)lp;
            }
        }
        // Real-space Ewald, each unordered pair once, spread evenly over the
        // lanes: pair p < NE (NE-1)/2 pairs electron i = p mod NE with
        // i + p / NE + 1 (mod NE) for the first NE floor((NE-1)/2) pairs and
        // i = p - that with i + NE/2 for the rest (even NE).  The minimum
        // image term is FP64; the other 26 images lie beyond L/2, where each
        // term is below erfc(alpha L/2)/(L/2), and are summed in FP32.
        double vreal = 0.0;
        ff vreal_ff = ff(0.0f);
        {
            TC* ps = Mr;                                  // the rows buffer is free again
            __syncwarp();
#pragma unroll
            for (int r = 0; r < 2; ++r) {
                const int j = lane + 32 * r;
                if (j < NE) { ps[3 * j] = P.x[r]; ps[3 * j + 1] = P.y[r]; ps[3 * j + 2] = P.z[r]; }
            }
            __syncwarp();
            constexpr int NPAIR = NE * (NE - 1) / 2, HALF = (NE - 1) / 2, FULL = NE * HALF;
            const float aLf = (float)((double)S.alpha * (double)S.L);
            const float rcu = (float)((double)S.rcut * (double)S.invL), rc2u = rcu * rcu;
            for (int p = lane; p < NPAIR; p += 32) {
                int i, j;
                if (p < FULL) {
                    i = p % NE;
                    j = i + p / NE + 1;
                } else {
                    i = p - FULL;
                    j = i + NE / 2;
                }
                if (j >= NE) j -= NE;
                const TC dx = min_img(ps[3 * i] - ps[3 * j], S), dy = min_img(ps[3 * i + 1] - ps[3 * j + 1], S),
                         dz = min_img(ps[3 * i + 2] - ps[3 * j + 2], S);
                if constexpr (std::is_same<TC, ff>::value) {
                    // float-float minimum-image term: no FP64 in this phase
                    const ff r = fsqrt(dx * dx + dy * dy + dz * dz);
                    if (r.hi > 1e-10f) vreal_ff += erfc_ff(S.alpha * r) / r;
                } else {
                    const double r = sqrt((double)dx * (double)dx + (double)dy * (double)dy + (double)dz * (double)dz);
                    if (r > 1e-10) vreal += erfc((double)S.alpha * r) / r;
                }
                if (S.real_images) {
                    // box units: the image shift is an exact integer, alpha L is
                    // exact in FP32 for the usual splittings, and sqrt and the
                    // quotient are correctly rounded, so the rounding of each
                    // term is unbiased; the sum is scaled by 1/L in FP64
                    const float sx = (float)((double)dx * (double)S.invL), sy = (float)((double)dy * (double)S.invL),
                                sz = (float)((double)dz * (double)S.invL);
                    float acc = 0.0f;
                    for (int ia = -1; ia <= 1; ++ia)
                        for (int ib = -1; ib <= 1; ++ib)
#pragma unroll
                            for (int ic = -1; ic <= 1; ++ic) {
                                if (!ia && !ib && !ic) continue;
                                const float ex = sx + (float)ia, ey = sy + (float)ib, ez = sz + (float)ic;
                                const float d2 = __fmaf_rn(ex, ex, __fmaf_rn(ey, ey, __fmul_rn(ez, ez)));
                                if (d2 < rc2u) {
                                    const float d = __fsqrt_rn(d2);
                                    acc += __fdiv_rn(erfcf(__fmul_rn(aLf, d)), d);
                                }
                            }
                    if constexpr (std::is_same<TC, ff>::value) vreal_ff += ff(acc) * S.invL;
                    else vreal += (double)acc * (double)S.invL;
                }
            }
        }
        // reciprocal Ewald: rho_k = sum_i e^{i k.r_i} over the half space of
        // integer vectors n (k = 2 pi n / L), visited in the order of the
        // host's weight table (nx, then ny, then nz ascending).  For each of
        // its electrons a lane keeps the running phase e^{i k.r}, advanced by
        // one complex multiply per step; one warp reduction per k.  Electrons
        // a lane does not own start from zero phase and contribute nothing.
        double vk = 0.0;
        {
            const double dk = 2.0 * M_PI / (double)S.L;
            const int K = S.kmax;
            TC exr[2], exi[2], eyr[2], eyi[2], ezr[2], ezi[2], ymr[2], ymi[2], zmr[2], zmi[2], pxr[2], pxi[2];
#pragma unroll
            for (int r = 0; r < 2; ++r) {
                const bool own = lane + 32 * r < NE;
                double s, c;
                sincos(dk * (double)P.x[r], &s, &c);
                exr[r] = own ? TC(c) : TC(0); exi[r] = own ? TC(s) : TC(0);
                sincos(dk * (double)P.y[r], &s, &c);
                eyr[r] = own ? TC(c) : TC(0); eyi[r] = own ? TC(s) : TC(0);
                sincos(dk * (double)P.z[r], &s, &c);
                ezr[r] = own ? TC(c) : TC(0); ezi[r] = own ? TC(s) : TC(0);
                // e^{-i K dk y}, e^{-i K dk z}: K multiplications by the conjugate
                ymr[r] = own ? TC(1) : TC(0); ymi[r] = TC(0);
                zmr[r] = own ? TC(1) : TC(0); zmi[r] = TC(0);
                for (int m = 0; m < K; ++m) {
                    TC t = ymr[r] * eyr[r] + ymi[r] * eyi[r];
                    ymi[r] = ymi[r] * eyr[r] - ymr[r] * eyi[r]; ymr[r] = t;
                    t = zmr[r] * ezr[r] + zmi[r] * ezi[r];
                    zmi[r] = zmi[r] * ezr[r] - zmr[r] * ezi[r]; zmr[r] = t;
                }
                pxr[r] = TC(1); pxi[r] = TC(0);
            }
            TC vkt = TC(0);
            int t = 0;
            for (int nx = 0; nx <= K; ++nx) {
                TC qr[2], qi[2];                              // e^{i (nx x + ny y) dk}, ny = -K
#pragma unroll
                for (int r = 0; r < 2; ++r) {
                    qr[r] = pxr[r] * ymr[r] - pxi[r] * ymi[r];
                    qi[r] = pxr[r] * ymi[r] + pxi[r] * ymr[r];
                }
                for (int ny = -K; ny <= K; ++ny) {
                    const int rest = K * K - nx * nx - ny * ny;
                    if (!(nx == 0 && ny < 0) && (S.kcube || rest >= 0)) {
                        TC tr[2], ti[2];                      // nz = -K
#pragma unroll
                        for (int r = 0; r < 2; ++r) {
                            tr[r] = qr[r] * zmr[r] - qi[r] * zmi[r];
                            ti[r] = qr[r] * zmi[r] + qi[r] * zmr[r];
                        }
                        // nz in chunks of four: the four lane partials of rho_k
                        // are reduced together (butterfly reduce-scatter: two
                        // exchanges at distance 16, one at 8, then a full
                        // reduction over the low three lane bits), after which
                        // lanes 0, 8, 16, 24 hold chunk values 0..3
                        const int vi = ((lane >> 4) & 1) * 2 + ((lane >> 3) & 1);
                        for (int nz0 = -K; nz0 <= K; nz0 += 4) {
                            TC pr[4], pim[4];
                            int tk[4];
                            bool ok4[4];
#pragma unroll
                            for (int j = 0; j < 4; ++j) {
                                const int nz = nz0 + j;
                                ok4[j] = nz <= K && !(nx == 0 && ny == 0 && nz <= 0) && (S.kcube || nz * nz <= rest);
                                tk[j] = t;
                                t += ok4[j] ? 1 : 0;
                                pr[j] = ok4[j] ? tr[0] + tr[1] : TC(0);
                                pim[j] = ok4[j] ? ti[0] + ti[1] : TC(0);
#pragma unroll
                                for (int r = 0; r < 2; ++r) {
                                    TC x = tr[r] * ezr[r] - ti[r] * ezi[r];
                                    ti[r] = tr[r] * ezi[r] + ti[r] * ezr[r];
                                    tr[r] = x;
                                }
                            }
                            const bool b4 = (lane & 16) != 0, b3 = (lane & 8) != 0;
                            TC wr[2], wi[2];
#pragma unroll
                            for (int h = 0; h < 2; ++h) {            // distance 16: keep v_h or v_{h+2}
                                const TC sr = b4 ? pr[h] : pr[h + 2], si = b4 ? pim[h] : pim[h + 2];
                                wr[h] = (b4 ? pr[h + 2] : pr[h]) + hshfl_xor(sr, 16);
                                wi[h] = (b4 ? pim[h + 2] : pim[h]) + hshfl_xor(si, 16);
                            }
                            const TC sr = b3 ? wr[0] : wr[1], si = b3 ? wi[0] : wi[1];   // distance 8
                            TC vr = (b3 ? wr[1] : wr[0]) + hshfl_xor(sr, 8);
                            TC vim = (b3 ? wi[1] : wi[0]) + hshfl_xor(si, 8);
#pragma unroll
                            for (int m = 4; m > 0; m >>= 1) {
                                vr += hshfl_xor(vr, m);
                                vim += hshfl_xor(vim, m);
                            }
                            const bool okv = vi == 0 ? ok4[0] : (vi == 1 ? ok4[1] : (vi == 2 ? ok4[2] : ok4[3]));
                            const int tv = vi == 0 ? tk[0] : (vi == 1 ? tk[1] : (vi == 2 ? tk[2] : tk[3]));
                            if ((lane & 7) == 0 && okv) vkt += kweight<TC>(static_cast<const KTable*>(a.kt), tv) * (vr * vr + vim * vim);
                        }
                    }
#pragma unroll
                    for (int r = 0; r < 2; ++r) {
                        TC x = qr[r] * eyr[r] - qi[r] * eyi[r];
                        qi[r] = qr[r] * eyi[r] + qi[r] * eyr[r];
                        qr[r] = x;
                    }
                }
#pragma unroll
                for (int r = 0; r < 2; ++r) {
                    TC x = pxr[r] * exr[r] - pxi[r] * exi[r];
                    pxi[r] = pxr[r] * exi[r] + pxi[r] * exr[r];
                    pxr[r] = x;
                }
            }
            vk = (double)hsum(vkt);
        }
        u = hsum(u);
        kin = hsum(kin);
        vreal = hsum(vreal + (double)vreal_ff);
        double V = vreal + vk + S.ksum_const + S.e_const;
        e_l = -0.5 * (double)kin + V;
        if (lane == 0) {
            int fl = 0;
            if (!ok) fl |= FLAG_SINGULAR;
            if (!isfinite(e_l)) fl |= FLAG_NONFINITE;
            if (fl) atomicOr(a.flags, fl);
            if (a.write_state) { a.log[w] = logdet + (double)u; a.sign[w] = 1; a.el[w] = e_l; }
        }
    }
    return act ? e_l : 0.0;
}

template <int WPB>
__device__ __forceinline__ void hwarp_block_partial(double v, double* partial, int slot) {
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

// Shared words per warp of a refresh launch: the orbital matrix rows for the
// determinant half, the positions for the energy half alone.
template <int NE, int NUP, int PART>
__host__ __device__ constexpr int hmeasure_warp_words() {
    return PART == 2 ? 3 * NE : 2 * (NUP > NE - NUP ? NUP : NE - NUP) * 32;
}

template <int NE, int NUP, class TC, class TS, int WPB, int PART = 0>
__global__ void __launch_bounds__(32 * WPB, PART == 2 ? 4 : 2) khw_measure(
    const SysH<TC>* __restrict__ Sg, const KTable* __restrict__ KT, const TS* __restrict__ gpos,
    TS* __restrict__ gdinv, double* __restrict__ glog, int* __restrict__ gsign, double* __restrict__ gel, int W,
    int Wcap, int write_state, double* __restrict__ out_grad, double* __restrict__ out_lap, double* partial,
    int* flags, float2* __restrict__ drows) {
    extern __shared__ __align__(16) unsigned char hsm[];
    __shared__ MeasureArgs<TS> args;
    SysH<TC>& S = *reinterpret_cast<SysH<TC>*>(hsm);
    TC* rows = reinterpret_cast<TC*>(hsm + ((sizeof(SysH<TC>) + 15) / 16) * 16);
    if (threadIdx.x == 0)
        args = MeasureArgs<TS>{gpos, gdinv, glog, gsign, gel, out_grad, out_lap, flags, drows, KT, W, Wcap,
                               write_state};
    load_sysh(&S, Sg, (int)sizeof(SysH<TC>));   // ends with a block barrier
    const volatile MeasureArgs<TS>& a = args;
    const int wib = threadIdx.x >> 5;
    const int w = blockIdx.x * WPB + wib;
    double e_l = khw_measure_walker<NE, NUP, TC, TS, PART>(
        S, a, rows + (size_t)wib * hmeasure_warp_words<NE, NUP, PART>(), w, w < W);
    if (PART != 1 && partial) hwarp_block_partial<WPB>(e_l, partial, blockIdx.x);
}

// Batched form (compute type TC, state written, per-tile E_L partials), one
// block per tile.
template <int NE, int NUP, class TC, class TS, int WPB, int PART = 0>
__global__ void __launch_bounds__(32 * WPB, PART == 2 ? 4 : 2) khwb_measure(const BatchTile* __restrict__ tiles,
                                                                         int ntiles, const BatchRec* __restrict__ recs,
                                                                         double* tile_partial) {
    extern __shared__ __align__(16) unsigned char hsm[];
    __shared__ MeasureArgs<TS> args;
    SysH<TC>& S = *reinterpret_cast<SysH<TC>*>(hsm);
    TC* rows = reinterpret_cast<TC*>(hsm + ((sizeof(SysH<TC>) + 15) / 16) * 16);
    if ((int)blockIdx.x >= ntiles) return;
    const int wib = threadIdx.x >> 5;
    const BatchTile tl = tiles[blockIdx.x];
    if (threadIdx.x == 0) args = measure_args<TS>(recs[tl.rec]);
    load_sysh(&S, static_cast<const SysH<TC>*>(recs[tl.rec].tab_d), (int)sizeof(SysH<TC>));   // ends with a barrier
    const volatile MeasureArgs<TS>& a = args;
    const int w = tl.w0 + wib;
    double e_l = khw_measure_walker<NE, NUP, TC, TS, PART>(
        S, a, rows + (size_t)wib * hmeasure_warp_words<NE, NUP, PART>(), w, w < a.W);
    if (PART != 1) hwarp_block_partial<WPB>(e_l, tile_partial, blockIdx.x);
}

int launch_sum_partials(const double* partial, int nblk, int nrows, double* out, cudaStream_t st);

template <int NE, int NUP>
struct HegShapeOps {
    static constexpr int NM = NUP > NE - NUP ? NUP : NE - NUP;
    static constexpr int WPB = 4;

    // Device copies: [SysH<T> | pad | KTable], cached per system and rebuilt
    // when the parameters change (HostSys::version).
    template <class T>
    static int table(const HostSys& hs, const SysH<T>** out, const KTable** kt = nullptr) {
        const int slot = std::is_same<T, double>::value ? 0 : (std::is_same<T, float>::value ? 1 : 2);
        const size_t off = ((sizeof(SysH<T>) + 255) / 256) * 256;
        if (!hs.dev_table[slot] || hs.dev_table_version[slot] != hs.version) {
            std::vector<unsigned char> buf(off + sizeof(KTable));
            SysH<T>* h = reinterpret_cast<SysH<T>*>(buf.data());
            KTable* k = reinterpret_cast<KTable*>(buf.data() + off);
            if (!fill_sysh<T>(hs, NE, NUP, *h, *k)) return 7;
            if (!hs.dev_table[slot] && cudaMalloc(&hs.dev_table[slot], buf.size()) != cudaSuccess) return 8;
            if (cudaMemcpy(hs.dev_table[slot], buf.data(), buf.size(), cudaMemcpyHostToDevice) != cudaSuccess) return 2;
            hs.dev_table_version[slot] = hs.version;
        }
        *out = static_cast<const SysH<T>*>(hs.dev_table[slot]);
        if (kt) *kt = reinterpret_cast<const KTable*>(static_cast<const unsigned char*>(hs.dev_table[slot]) + off);
        return 0;
    }

    // ---- batched launches ---------------------------------------------------
    // tab_s: the sweep table (walker precision); tab_d: the refresh table
    // (FP64 for FP64 walkers, float-float for FP32 walkers).
    static int batch_tables(const HostSys& hs, int prec, BatchRec& r) {
        const KTable* kt;
        if (prec == 0) {
            const SysH<double>* d;
            int rc = table<double>(hs, &d, &kt);
            if (rc) return rc;
            r.tab_d = r.tab_s = d;
            r.ktab = kt;
            return 0;
        }
        const SysH<ff>* m;
        const SysH<float>* f;
        int rc = table<ff>(hs, &m, &kt);
        if (!rc) rc = table<float>(hs, &f);
        if (rc) return rc;
        r.tab_d = m;
        r.tab_s = f;
        r.ktab = kt;
        return 0;
    }

    template <class T, int MOVE>
    static int batch_sweep_t(const BatchClass& bc, const BatchCtl* ctl, cudaStream_t st, int* occ) {
        auto kern = khwb_sweep<NE, NUP, T, MOVE, WPB>;
        const size_t smem = WPB * hsweep_warp_bytes<NM, T>();
        static bool attr = false;
        if (!attr) {
            if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
                return 2;
            cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
            attr = true;
        }
        if (occ) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, kern, 32 * WPB, smem) == cudaSuccess ? 0 : 2;
        if (bc.ntiles == 0) return 0;
        kern<<<bc.ntiles, 32 * WPB, smem, st>>>(bc.tiles, bc.ntiles, bc.recs, ctl);
        ++g_launch_count;
        return cudaGetLastError() == cudaSuccess ? 0 : 2;
    }

    // The electron-gas sweep has no fixed-node form: batches of it run VMC only.
    static int batch_sweep(const BatchClass& bc, int mk, const BatchCtl* ctl, cudaStream_t st, int* occ = nullptr) {
        if (mk == MOVE_ONE_GAUSS)
            return bc.prec == 0 ? batch_sweep_t<double, MOVE_ONE_GAUSS>(bc, ctl, st, occ)
                                : batch_sweep_t<float, MOVE_ONE_GAUSS>(bc, ctl, st, occ);
        if (mk == MOVE_ONE_DRIFT)
            return bc.prec == 0 ? batch_sweep_t<double, MOVE_ONE_DRIFT>(bc, ctl, st, occ)
                                : batch_sweep_t<float, MOVE_ONE_DRIFT>(bc, ctl, st, occ);
        return 7;
    }

    template <class TC, class TS, int PART>
    static size_t measure_smem() {
        return ((sizeof(SysH<TC>) + 15) / 16) * 16 + sizeof(TC) * WPB * hmeasure_warp_words<NE, NUP, PART>();
    }

    template <class TC, class TS, int PART>
    static int batch_measure_t(const BatchClass& bc, cudaStream_t st, int* occ) {
        const size_t smem = measure_smem<TC, TS, PART>();
        auto kern = khwb_measure<NE, NUP, TC, TS, WPB, PART>;
        static bool attr = false;
        if (!attr) { cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); attr = true; }
        if (occ) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, kern, 32 * WPB, smem) == cudaSuccess ? 0 : 2;
        if (bc.ntiles == 0) return 0;
        kern<<<bc.ntiles, 32 * WPB, smem, st>>>(bc.tiles, bc.ntiles, bc.recs, bc.tile_partial);
        ++g_launch_count;
        return cudaGetLastError() == cudaSuccess ? 0 : 2;
    }

    // FP32 walker sets (which carry the refresh scratch) refresh in two
    // launches, FP64 ones in one; the occupancy reported is the lower of the
    // two halves'.
    static int batch_measure(const BatchClass& bc, cudaStream_t st, int* occ = nullptr) {
        if (bc.prec == 0) return batch_measure_t<double, double, 0>(bc, st, occ);
        if (occ) {
            int o1 = 0, o2 = 0;
            int rc = batch_measure_t<ff, float, 1>(bc, st, &o1);
            if (!rc) rc = batch_measure_t<ff, float, 2>(bc, st, &o2);
            *occ = o1 < o2 ? o1 : o2;
            return rc;
        }
        int rc = batch_measure_t<ff, float, 1>(bc, st, nullptr);
        return rc ? rc : batch_measure_t<ff, float, 2>(bc, st, nullptr);
    }

    static int init(const HostSys& hs, DevWalkers& dw, uint64_t seed, cudaStream_t st) {
        const SysH<double>* S;
        int rc = table<double>(hs, &S);
        if (rc) return rc;
        int n = NE * dw.W, tpb = 256;
        if (dw.prec == 0) khw_init<double><<<(n + tpb - 1) / tpb, tpb, 0, st>>>(S, (double*)dw.pos, NE, dw.W, dw.Wcap, seed);
        else khw_init<float><<<(n + tpb - 1) / tpb, tpb, 0, st>>>(S, (float*)dw.pos, NE, dw.W, dw.Wcap, seed);
        ++g_launch_count;
        return cudaGetLastError() == cudaSuccess ? 0 : 2;
    }

    template <class TC, class TS, int PART>
    static int launch_measure_part(const SysH<TC>* S, const KTable* KT, DevWalkers& dw, bool ws, const MeasureOut& out,
                                   double* partial, int nb, cudaStream_t st) {
        const size_t smem = measure_smem<TC, TS, PART>();
        auto kern = khw_measure<NE, NUP, TC, TS, WPB, PART>;
        static bool attr = false;
        if (!attr) { cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); attr = true; }
        kern<<<nb, 32 * WPB, smem, st>>>(S, KT, (const TS*)dw.pos, (TS*)dw.dinv, dw.logabs, dw.sign, dw.el, dw.W,
                                         dw.Wcap, ws ? 1 : 0, out.grad, out.lap, partial, dw.flags, dw.rows);
        ++g_launch_count;
        return cudaGetLastError() == cudaSuccess ? 0 : 2;
    }

    template <class TC, class TS>
    static int measure2(const HostSys& hs, DevWalkers& dw, bool ws, const MeasureOut& out, cudaStream_t st) {
        const SysH<TC>* S;
        const KTable* KT;
        int rc = table<TC>(hs, &S, &KT);
        if (rc) return rc;
        int nb = (dw.W + WPB - 1) / WPB;
        double* partial = (ws && dw.partial && dw.partial_cap >= 2 * nb + 1) ? dw.partial : nullptr;
        bool two = false;
        if constexpr (std::is_same<TC, ff>::value) two = ws && dw.rows && !out.grad && !out.lap;
        if (two) {
            if constexpr (std::is_same<TC, ff>::value) {
                rc = launch_measure_part<TC, TS, 1>(S, KT, dw, ws, out, nullptr, nb, st);
                if (!rc) rc = launch_measure_part<TC, TS, 2>(S, KT, dw, ws, out, partial, nb, st);
            }
        } else {
            rc = launch_measure_part<TC, TS, 0>(S, KT, dw, ws, out, partial, nb, st);
        }
        if (rc) return rc;
        if (!partial) return 0;
        return launch_sum_partials(partial, nb, 1, dw.partial + dw.partial_cap - 1, st);
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
        const SysH<T>* S;
        int rc = table<T>(hs, &S);
        if (rc) return rc;
        int nb = (dw.W + WPB - 1) / WPB;
        auto kern = khw_sweep<NE, NUP, T, MOVE, WPB>;
        const size_t smem = WPB * hsweep_warp_bytes<NM, T>();
        static bool attr = false;
        if (!attr) {
            if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
                return 2;
            cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
            attr = true;
        }
        kern<<<nb, 32 * WPB, smem, st>>>(S, (T*)dw.pos, (T*)dw.dinv, dw.W, dw.Wcap, n, s0, (T)step, (T)tau, (T)maxd,
                                         seed, dw.acc, dw.flags);
        ++g_launch_count;
        return cudaGetLastError() == cudaSuccess ? 0 : 2;
    }

    static int sweep(const HostSys& hs, DevWalkers& dw, int mk, int n, uint64_t s0, double step, double tau,
                     double maxd, uint64_t seed, cudaStream_t st) {
        if (dw.fixed_node) return 7;     // complex determinants have no nodal surface to fix
        if (mk == MOVE_ONE_GAUSS)
            return dw.prec == 0 ? sweep_t<double, MOVE_ONE_GAUSS>(hs, dw, n, s0, step, tau, maxd, seed, st)
                                : sweep_t<float, MOVE_ONE_GAUSS>(hs, dw, n, s0, step, tau, maxd, seed, st);
        if (mk == MOVE_ONE_DRIFT)
            return dw.prec == 0 ? sweep_t<double, MOVE_ONE_DRIFT>(hs, dw, n, s0, step, tau, maxd, seed, st)
                                : sweep_t<float, MOVE_ONE_DRIFT>(hs, dw, n, s0, step, tau, maxd, seed, st);
        return 7;
    }
};

}  // namespace qmc

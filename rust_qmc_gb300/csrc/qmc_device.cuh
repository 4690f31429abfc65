// qmc_device.cuh -- device-side system tables and the per-walker building
// blocks of the Slater-Jastrow walker path: counter-based RNG, AO->MO
// evaluation, Jastrow pair terms, Gauss-Jordan inverse, Sherman-Morrison
// update.  One thread owns one walker; every per-walker array is indexed with
// compile-time indices so it stays in registers or in the thread's own
// shared-memory column.
#pragma once
#include <cstdint>
#include <type_traits>
#include <utility>
#include <cuda_runtime.h>
#include "qmc_ff.cuh"

namespace qmc {

enum { BASIS_GTO = 0, BASIS_STO = 1 };
enum { JAS_NONE = 0, JAS_PADE_F = 1, JAS_PADE_EEN = 2 };
enum { MOVE_ALL_GAUSS = 0, MOVE_ALL_BOX = 1, MOVE_ONE_GAUSS = 2, MOVE_ONE_DRIFT = 3 };
enum { TAG_PROPOSE = 1, TAG_ACCEPT = 2, TAG_INIT = 3, TAG_BRANCH = 4 };
enum { FLAG_SINGULAR = 1, FLAG_NONFINITE = 2, FLAG_TIMEOUT = 8 };

// Compile-time basis layout of the 9-function CH4 workload: shell s sits on
// nucleus nuc(s), has np(s) primitives and is kind 1 (one s AO) or kind 2
// (an s AO plus a p triplet sharing exponents).  Shells are ordered by
// nucleus; AO and primitive indices are the prefix sums the host uses.
struct LayoutCH4Min {
    static constexpr int NSHELL = 6;
    __host__ __device__ static constexpr int nuc(int s) { return s < 2 ? 0 : s - 1; }
    __host__ __device__ static constexpr int np(int) { return 3; }
    __host__ __device__ static constexpr int kind(int s) { return s == 1 ? 2 : 1; }
    __host__ __device__ static constexpr int p0(int s) { return 3 * s; }
    __host__ __device__ static constexpr int ao0(int s) { return s < 2 ? s : s + 3; }
};

template <int NE_, int NUP_, int NNUC_, int NSH_, int NAO_, int NPRIM_, int BASIS_, int JAS_, int NROT_,
          class LAYOUT_ = void>
struct ShapeT {
    static constexpr int NE = NE_, NUP = NUP_, NDN = NE_ - NUP_, NNUC = NNUC_;
    static constexpr int NSH = NSH_, NAO = NAO_, NPRIM = NPRIM_, BASIS = BASIS_, JAS = JAS_;
    static constexpr int NROT = NROT_;
    static constexpr int NMAX = NUP_ > (NE_ - NUP_) ? NUP_ : (NE_ - NUP_);
    using Layout = LAYOUT_;
};

// H2 LCAO (src/systems/hydrogen.rs:28-35): 2 Slater 1s AOs, 1 up + 1 down.
using ShapeH2 = ShapeT<2, 1, 2, 2, 2, 2, BASIS_STO, JAS_PADE_F, 1>;
// Li atom (src/systems/lithium.rs, src/main.rs:37-48): STO-7G 1s/2s, 2 up + 1 down.
using ShapeLi = ShapeT<3, 2, 1, 1, 2, 8, BASIS_STO, JAS_PADE_F, 1>;
// CH4 (src/systems/methane.rs:600-776): up to 17 Gaussian AOs, 5 up + 5 down.
using ShapeCH4 = ShapeT<10, 5, 5, 12, 17, 28, BASIS_GTO, JAS_PADE_EEN, 4>;
// The 9-function CH4 workload with its basis layout fixed at compile time.
using ShapeCH4Min = ShapeT<10, 5, 5, 6, 9, 18, BASIS_GTO, JAS_PADE_EEN, 4, LayoutCH4Min>;

template <class SH, class T>
struct SysT {
    T nuc[SH::NNUC][3];
    T Z[SH::NNUC];
    T enA[SH::NNUC];          // A_species * Z_I (e-n Jastrow amplitude)
    T enB[SH::NNUC];          // B_species
    T Aspec[SH::NNUC];        // A_species (unscaled)
    int species[SH::NNUC];
    T F, invF;                // Pade-F parameter and 1/F
    T b_ee[2], a_ee[2];       // [0] antiparallel, [1] parallel
    T qa;                     // Jastrow2 gradient prefactor quirk (F or 1)
    int quirk_lap;            // Jastrow2 Laplacian quirk
    T v_nn;
    int n_rot;
    int sh_start[SH::NNUC + 1];
    int sh_p0[SH::NSH], sh_np[SH::NSH];
    int sh_s0[SH::NSH], sh_s1[SH::NSH], sh_p[SH::NSH];
    T pexp[SH::NPRIM];
    T pexp2[SH::NPRIM];             // -pexp log2(e): FP32 Gaussians as 2^(pexp2 r^2)
    T cs0[SH::NPRIM], cs1[SH::NPRIM], cp[SH::NPRIM];
    int ppow[SH::NPRIM];
    T C[2][SH::NAO][SH::NMAX];      // [sector][internal AO][column]
    T dC[SH::NROT][SH::NAO];        // d phi / d theta rows
    int rot_col[SH::NROT][2];       // column of the rotated MO in each sector (-1 none)
    T init_sigma;
    int init_nuc[SH::NE];           // internal electron order
    int perm[SH::NE];               // internal -> caller electron index
};

template <int J>
struct IntC { static constexpr int value = J; };
template <int N, class F, int... Is>
__device__ __forceinline__ void unroll_impl(F&& f, std::integer_sequence<int, Is...>) { (f(IntC<Is>{}), ...); }
// f(IntC<0>{}), ..., f(IntC<N-1>{}) with compile-time indices.
template <int N, class F>
__device__ __forceinline__ void static_for(F&& f) { unroll_impl<N>(f, std::make_integer_sequence<int, N>{}); }

// ---------------------------------------------------------------------------
// Math helpers (float paths use the hardware approximations).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double fexp(double x) { return exp(x); }
__device__ __forceinline__ float fexp(float x) { return __expf(x); }
__device__ __forceinline__ double flog(double x) { return log(x); }
__device__ __forceinline__ float flog(float x) { return __logf(x); }
__device__ __forceinline__ double fsqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float fsqrt(float x) { return sqrtf(x); }
// Double-precision reciprocal and reciprocal square root: single-precision
// hardware seed refined by one Newton-Raphson step, y1 = y0 (2 - x y0) and
// y1 = y0 (3 - x y0^2) / 2, which squares the seed's ~2^-22 relative error
// to ~1e-14.  Arguments are positive and within single-precision range here.
__device__ __forceinline__ double frcp(double x) {
    double y = (double)__fdividef(1.0f, (float)x);
    double e = fma(-x, y, 1.0);
    return fma(e, y, y);
}
__device__ __forceinline__ float frcp(float x) { return __fdividef(1.0f, x); }
// 2^x by the PTX approximate base-2 exponential (flush-to-zero).
__device__ __forceinline__ float ex2_approx(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al., SC'11) and the stream layout of include/qmc.h.
// ---------------------------------------------------------------------------
struct U4 { uint32_t x, y, z, w; };
__host__ __device__ __forceinline__ U4 philox(U4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        // one 32 x 32 -> 64-bit product per multiplier (a single wide
        // multiply on the device)
        uint64_t p0 = (uint64_t)0xD2511F53u * c.x, p1 = (uint64_t)0xCD9E8D57u * c.z;
        uint32_t lo0 = (uint32_t)p0, hi0 = (uint32_t)(p0 >> 32);
        uint32_t lo1 = (uint32_t)p1, hi1 = (uint32_t)(p1 >> 32);
        U4 n;
        n.x = hi1 ^ c.y ^ k0;
        n.y = lo1;
        n.z = hi0 ^ c.w ^ k1;
        n.w = lo0;
        c = n;
    }
    return c;
}
__device__ __forceinline__ U4 rng_draw(uint64_t seed, uint32_t walker, uint64_t step, uint32_t sub, uint32_t tag) {
    U4 c{walker, (uint32_t)step, sub, tag | ((uint32_t)((step >> 32) & 0xFFFFu) << 16)};
    return philox(c, (uint32_t)seed, (uint32_t)(seed >> 32));
}
// A single-electron move takes one Philox call: four 24-bit uniforms feed two
// Box-Muller pairs (three displacement components are used) and the top
// bytes of words 0-2 form the 24-bit acceptance uniform.
__device__ __forceinline__ double u24(uint32_t k, double) { return ((double)k + 0.5) * (1.0 / 16777216.0); }
__device__ __forceinline__ float u24(uint32_t k, float) { return ((float)k + 0.5f) * (1.0f / 16777216.0f); }
template <class T>
struct MoveDraw { T n0, n1, n2, uacc; };
__device__ __forceinline__ void bm24(uint32_t a, uint32_t b, double& n0, double& n1) {
    double r = sqrt(-2.0 * log(u24(a, 0.0)));
    double s, c;
    sincospi(2.0 * u24(b, 0.0), &s, &c);
    n0 = r * c; n1 = r * s;
}
__device__ __forceinline__ void bm24(uint32_t a, uint32_t b, float& n0, float& n1) {
    float r = sqrtf(-2.0f * __logf(u24(a, 0.0f)));
    float s, c;
    __sincosf(6.28318530717958647f * u24(b, 0.0f), &s, &c);
    n0 = r * c; n1 = r * s;
}
__device__ __forceinline__ double to_u01(uint32_t x, double) { return ((double)x + 0.5) * (1.0 / 4294967296.0); }
__device__ __forceinline__ float to_u01(uint32_t x, float) { return ((float)(x >> 8) + 0.5f) * (1.0f / 16777216.0f); }
__device__ __forceinline__ void bm(uint32_t a, uint32_t b, double& n0, double& n1) {
    double r = sqrt(-2.0 * log(to_u01(a, 0.0)));
    double s, c;
    sincospi(2.0 * to_u01(b, 0.0), &s, &c);
    n0 = r * c; n1 = r * s;
}
__device__ __forceinline__ void bm(uint32_t a, uint32_t b, float& n0, float& n1) {
    float r = sqrtf(-2.0f * __logf(to_u01(a, 0.0f)));
    float s, c;
    __sincosf(6.28318530717958647f * to_u01(b, 0.0f), &s, &c);
    n0 = r * c; n1 = r * s;
}

template <class T>
__device__ __forceinline__ MoveDraw<T> move_draw(uint64_t seed, uint32_t walker, uint64_t step, uint32_t e) {
    U4 x = rng_draw(seed, walker, step, e, TAG_PROPOSE);
    MoveDraw<T> d;
    T n3;
    bm24(x.x & 0xFFFFFFu, x.y & 0xFFFFFFu, d.n0, d.n1);
    bm24(x.z & 0xFFFFFFu, x.w & 0xFFFFFFu, d.n2, n3);
    uint32_t ua = (x.x >> 24) | ((x.y >> 24) << 8) | ((x.z >> 24) << 16);
    d.uacc = u24(ua, T(0));
    return d;
}

// Warp-per-walker sweeps: lane i draws the proposal of electron e0 + i of
// the sector (i < ns <= 32) once per sweep, and proposal q reads draw q with
// a shuffle -- the same counters, so the same stream as one draw per move.
template <class T>
__device__ __forceinline__ MoveDraw<T> sector_draws(uint64_t seed, uint32_t walker, uint64_t step, int e0, int ns,
                                                    int lane) {
    MoveDraw<T> d{T(0), T(0), T(0), T(0)};
    if (lane < ns) d = move_draw<T>(seed, walker, step, (uint32_t)(e0 + lane));
    return d;
}
template <class T>
__device__ __forceinline__ MoveDraw<T> draw_of(const MoveDraw<T>& d, int q) {
    MoveDraw<T> r;
    r.n0 = __shfl_sync(0xffffffffu, d.n0, q);
    r.n1 = __shfl_sync(0xffffffffu, d.n1, q);
    r.n2 = __shfl_sync(0xffffffffu, d.n2, q);
    r.uacc = __shfl_sync(0xffffffffu, d.uacc, q);
    return r;
}

// ---------------------------------------------------------------------------
// Orbital evaluation: phi_k(r) = sum_a C[sig][a][k] chi_a(r) for the NS
// columns of sector SIG, optionally with gradients (MODE >= 1) and
// Laplacians (MODE >= 2), and NR extra rows (rotation derivatives, values).
// Shells are grouped by nucleus; each shell's primitive exponentials are
// computed once and shared by its s-type AOs and p triplet
// (src/systems/methane.rs:498-590 for Gaussians, src/wavefunction/slater.rs:
// 91-145 for Slater-type radial functions).
// ---------------------------------------------------------------------------
// Gaussian primitive p at squared distance r2: exp(-alpha r^2); FP32 uses
// the pre-scaled exponent and one base-2 exponential.
template <class SH, class T>
__device__ __forceinline__ T gauss_prim(const SysT<SH, T>& S, int p, T r2) { return fexp(-S.pexp[p] * r2); }
template <class SH>
__device__ __forceinline__ float gauss_prim(const SysT<SH, float>& S, int p, float r2) {
    return ex2_approx(S.pexp2[p] * r2);
}

// MODE 3 adds the gradients and Laplacians of the NR rotation rows (the
// parameter derivatives of the local energy need them).
template <class SH, class T, int SIG, int MODE, int NR>
struct MOEval {
    static constexpr int NS = SIG == 0 ? SH::NUP : SH::NDN;
    static constexpr int NRD = (MODE >= 3 && NR > 0) ? NR : 1;
    T v[SH::NMAX], gx[SH::NMAX], gy[SH::NMAX], gz[SH::NMAX], l[SH::NMAX];
    T dv[NR > 0 ? NR : 1];
    T dgx[NRD], dgy[NRD], dgz[NRD], dl[NRD];

    __device__ __forceinline__ void add(const SysT<SH, T>& S, int a, T chi, T ax, T ay, T az, T la) {
#pragma unroll
        for (int k = 0; k < NS; ++k) {
            T c = S.C[SIG][a][k];
            v[k] += c * chi;
            if (MODE >= 1) { gx[k] += c * ax; gy[k] += c * ay; gz[k] += c * az; }
            if (MODE >= 2) l[k] += c * la;
        }
#pragma unroll
        for (int q = 0; q < NR; ++q) {
            const T c = S.dC[q][a];
            dv[q] += c * chi;
            if (MODE >= 3) { dgx[q] += c * ax; dgy[q] += c * ay; dgz[q] += c * az; dl[q] += c * la; }
        }
    }

    // GTO shell: accumulate one shell's s AO (index a) and optional p triplet.
    __device__ __forceinline__ void gto_shell(const SysT<SH, T>& S, int a, bool has_p, T a0, T b0, T c0, T ap,
                                              T bp, T cpp, T dx, T dy, T dz, T r2) {
        add(S, a, a0, -2 * b0 * dx, -2 * b0 * dy, -2 * b0 * dz, -6 * b0 + 4 * r2 * c0);
        if (has_p) {
            T lp = -10 * bp + 4 * r2 * cpp;
            add(S, a + 1, dx * ap, dx * (-2 * bp * dx) + ap, dx * (-2 * bp * dy), dx * (-2 * bp * dz), dx * lp);
            add(S, a + 2, dy * ap, dy * (-2 * bp * dx), dy * (-2 * bp * dy) + ap, dy * (-2 * bp * dz), dy * lp);
            add(S, a + 3, dz * ap, dz * (-2 * bp * dx), dz * (-2 * bp * dy), dz * (-2 * bp * dz) + ap, dz * lp);
        }
    }

    // only_nuc >= 0 restricts the sum to AOs centred on that nucleus.
    __device__ __forceinline__ void run(const SysT<SH, T>& S, T x, T y, T z, int only_nuc = -1) {
#pragma unroll
        for (int k = 0; k < SH::NMAX; ++k) { v[k] = 0; gx[k] = 0; gy[k] = 0; gz[k] = 0; l[k] = 0; }
#pragma unroll
        for (int q = 0; q < (NR > 0 ? NR : 1); ++q) dv[q] = 0;
#pragma unroll
        for (int q = 0; q < NRD; ++q) { dgx[q] = 0; dgy[q] = 0; dgz[q] = 0; dl[q] = 0; }
        if constexpr (!std::is_void<typename SH::Layout>::value) {
            using LY = typename SH::Layout;
#pragma unroll
            for (int sh = 0; sh < LY::NSHELL; ++sh) {
                const int I = LY::nuc(sh), p0 = LY::p0(sh), a = LY::ao0(sh);
                const bool has_p = LY::kind(sh) == 2;
                if (only_nuc >= 0 && only_nuc != I) continue;
                T dx = x - S.nuc[I][0], dy = y - S.nuc[I][1], dz = z - S.nuc[I][2];
                T r2 = dx * dx + dy * dy + dz * dz;
                T a0 = 0, b0 = 0, c0 = 0, ap = 0, bp = 0, cpp = 0;
#pragma unroll
                for (int p = p0; p < p0 + LY::np(sh); ++p) {
                    T al = S.pexp[p];
                    T e = gauss_prim(S, p, r2);
                    T e0 = S.cs0[p] * e;
                    a0 += e0;
                    if (MODE >= 1) b0 += al * e0;
                    if (MODE >= 2) c0 += al * al * e0;
                    if (has_p) {
                        T ep = S.cp[p] * e;
                        ap += ep;
                        if (MODE >= 1) bp += al * ep;
                        if (MODE >= 2) cpp += al * al * ep;
                    }
                }
                gto_shell(S, a, has_p, a0, b0, c0, ap, bp, cpp, dx, dy, dz, r2);
            }
        } else {
            run_tables(S, x, y, z, only_nuc);
        }
    }

    // Table-driven shells (runtime shell and primitive counts).
    __device__ __forceinline__ void run_tables(const SysT<SH, T>& S, T x, T y, T z, int only_nuc) {
#pragma unroll
        for (int I = 0; I < SH::NNUC; ++I) {
            if (only_nuc >= 0 && only_nuc != I) continue;
            T dx = x - S.nuc[I][0], dy = y - S.nuc[I][1], dz = z - S.nuc[I][2];
            T r2 = dx * dx + dy * dy + dz * dz;
            for (int sh = S.sh_start[I]; sh < S.sh_start[I + 1]; ++sh) {
                int p0 = S.sh_p0[sh], p1 = p0 + S.sh_np[sh];
                if (SH::BASIS == BASIS_GTO) {
                    T a0 = 0, a1 = 0, ap = 0, b0 = 0, b1 = 0, bp = 0, c0 = 0, c1 = 0, cpp = 0;
                    for (int p = p0; p < p1; ++p) {
                        T al = S.pexp[p];
                        T e = gauss_prim(S, p, r2);
                        T e0 = S.cs0[p] * e, e1 = S.cs1[p] * e, ep = S.cp[p] * e;
                        a0 += e0; a1 += e1; ap += ep;
                        if (MODE >= 1) { b0 += al * e0; b1 += al * e1; bp += al * ep; }
                        if (MODE >= 2) { c0 += al * al * e0; c1 += al * al * e1; cpp += al * al * ep; }
                    }
                    int s0 = S.sh_s0[sh], s1 = S.sh_s1[sh], pa = S.sh_p[sh];
                    if (s0 >= 0) add(S, s0, a0, -2 * b0 * dx, -2 * b0 * dy, -2 * b0 * dz, -6 * b0 + 4 * r2 * c0);
                    if (s1 >= 0) add(S, s1, a1, -2 * b1 * dx, -2 * b1 * dy, -2 * b1 * dz, -6 * b1 + 4 * r2 * c1);
                    if (pa >= 0) {
                        T lp = -10 * bp + 4 * r2 * cpp;
                        // chi = x_m R(r): grad = x_m (-2 R1 dr) + e_m R0, lap = x_m(-10 R1 + 4 r^2 R2)
                        add(S, pa + 0, dx * ap, dx * (-2 * bp * dx) + ap, dx * (-2 * bp * dy), dx * (-2 * bp * dz), dx * lp);
                        add(S, pa + 1, dy * ap, dy * (-2 * bp * dx), dy * (-2 * bp * dy) + ap, dy * (-2 * bp * dz), dy * lp);
                        add(S, pa + 2, dz * ap, dz * (-2 * bp * dx), dz * (-2 * bp * dy), dz * (-2 * bp * dz) + ap, dz * lp);
                    }
                } else {
                    // Slater-type: R(d) = sum c d^n e^{-zeta d}
                    T d = fsqrt(r2);
                    T id = d > 0 ? frcp(d) : T(0);
                    T v0 = 0, v1 = 0, d0 = 0, d1 = 0, l0 = 0, l1 = 0;
                    for (int p = p0; p < p1; ++p) {
                        T zt = S.pexp[p];
                        int n = S.ppow[p];
                        T dn = 1;
                        for (int t = 0; t < n; ++t) dn *= d;
                        T dn1 = dn * id, dn2 = dn1 * id;
                        T e = fexp(-zt * d);
                        T nf = (T)n;
                        T val = dn * e;
                        T rd = e * (-zt * dn + nf * dn1);
                        T lap = e * (zt * zt * dn - 2 * zt * nf * dn1 + nf * (nf - 1) * dn2) + 2 * rd * id;
                        v0 += S.cs0[p] * val; v1 += S.cs1[p] * val;
                        d0 += S.cs0[p] * rd;  d1 += S.cs1[p] * rd;
                        l0 += S.cs0[p] * lap; l1 += S.cs1[p] * lap;
                    }
                    int s0 = S.sh_s0[sh], s1 = S.sh_s1[sh];
                    T ux = dx * id, uy = dy * id, uz = dz * id;
                    if (d == 0) { l0 = 0; l1 = 0; }
                    if (s0 >= 0) add(S, s0, v0, d0 * ux, d0 * uy, d0 * uz, l0);
                    if (s1 >= 0) add(S, s1, v1, d1 * ux, d1 * uy, d1 * uz, l1);
                }
            }
        }
    }
};

// ---------------------------------------------------------------------------
// Jastrow pair functions.  Returns u, u'(r) and u'' + 2u'/r.
// PADE_F: u = -F/(2(1+r/F))   (src/correlation/jastrow.rs:30-53, 85-125)
// PADE_EEN e-e: u = a r/(1+b r); e-n: u = -A r/(1+B r)   (:218-321)
// ---------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ T frsqrt(T x);
template <>
__device__ __forceinline__ double frsqrt<double>(double x) {
    double y = (double)rsqrtf((float)x);
    double e = fma(-x * y, y, 1.0);
    return fma(0.5 * e, y, y);
}
template <>
__device__ __forceinline__ float frsqrt<float>(float x) { return rsqrtf(x); }

// Distance and reciprocal distance from a squared distance (one rsqrt).
template <class T>
__device__ __forceinline__ void dist(T r2, T& d, T& rinv) {
    rinv = r2 > T(0) ? frsqrt(r2) : T(0);
    d = r2 * rinv;
}

// upr = u'(r)/r, lt = u'' + 2u'/r.  rinv = 1/r (0 at r = 0).
template <class T>
__device__ __forceinline__ void pade_f(T F, T invF, T d, T rinv, T& u, T& upr, T& lt) {
    T inv = frcp(1 + d * invF);
    u = -F * T(0.5) * inv;
    T up = T(0.5) * inv * inv;
    upr = up * rinv;
    lt = inv * inv * inv * rinv;
}
template <class T>
__device__ __forceinline__ void pade_ab(T a, T b, T d, T rinv, T& u, T& upr, T& lt) {
    T inv = frcp(1 + b * d);
    u = a * d * inv;
    T up = a * inv * inv;
    upr = up * rinv;
    lt = 2 * up * rinv - 2 * a * b * inv * inv * inv;
}

// ---------------------------------------------------------------------------
// Gauss-Jordan inverse with partial pivoting (restates the LU-based
// determinant/try_inverse the reference calls at src/systems/methane.rs:
// 828-829).  A is destroyed; Ainv = A^-1.  Row swaps use selects so that
// all indices stay compile-time.
// ---------------------------------------------------------------------------
// on_pivot(|pivot|) receives each pivot magnitude for the determinant.
template <int N, class T, class OnPivot>
__device__ __forceinline__ bool gj_inverse_core(T (&A)[N][N], T (&Ainv)[N][N], int& sign, OnPivot on_pivot) {
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
        for (int j = 0; j < N; ++j) Ainv[i][j] = (i == j) ? T(1) : T(0);
    sign = 1;
    bool ok = true;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        int p = k;
        T best = fabs(A[k][k]);
#pragma unroll
        for (int i = k + 1; i < N; ++i) {
            T a = fabs(A[i][k]);
            if (a > best) { best = a; p = i; }
        }
#pragma unroll
        for (int i = k + 1; i < N; ++i) {
            bool sw = (i == p);
#pragma unroll
            for (int j = 0; j < N; ++j) {
                T a = A[k][j], b = A[i][j];
                A[k][j] = sw ? b : a; A[i][j] = sw ? a : b;
                T c = Ainv[k][j], d = Ainv[i][j];
                Ainv[k][j] = sw ? d : c; Ainv[i][j] = sw ? c : d;
            }
        }
        if (p != k) sign = -sign;
        T piv = A[k][k];
        if (!(piv != T(0))) { ok = false; piv = T(1); }
        if (piv < 0) sign = -sign;
        on_pivot(fabs(piv));
        T ip = T(1) / piv;
#pragma unroll
        for (int j = 0; j < N; ++j) { A[k][j] *= ip; Ainv[k][j] *= ip; }
#pragma unroll
        for (int i = 0; i < N; ++i) {
            if (i == k) continue;
            T f = A[i][k];
#pragma unroll
            for (int j = 0; j < N; ++j) { A[i][j] -= f * A[k][j]; Ainv[i][j] -= f * Ainv[k][j]; }
        }
    }
    return ok;
}

template <int N, class T>
__device__ __forceinline__ bool gj_inverse(T (&A)[N][N], T (&Ainv)[N][N], double& logdet, int& sign) {
    logdet = 0.0;
    return gj_inverse_core<N, T>(A, Ainv, sign, [&](T p) { logdet += log((double)p); });
}

// Float-float form: |det| accumulated as a rescaled product (one logarithm
// per caller instead of one FP64 logarithm per pivot).
template <int N>
__device__ __forceinline__ bool gj_inverse_prod(ff (&A)[N][N], ff (&Ainv)[N][N], ff& pm, int& pe, int& sign) {
    return gj_inverse_core<N, ff>(A, Ainv, sign, [&](ff p) {
        pm = pm * p;
        ff_rescale(pm, pe);
    });
}

// Neumaier-compensated pair (s, c): value = s + c.
struct Comp { double s, c; };
__device__ __forceinline__ Comp comp_add(Comp a, Comp b) {
    double s = a.s + b.s;
    double e = fabs(a.s) >= fabs(b.s) ? (a.s - s) + b.s : (b.s - s) + a.s;
    return {s, a.c + b.c + e};
}

// Compensated sum of v over the block's TPB threads into partial[2 slot],
// partial[2 slot + 1] (a fixed-order tree; every thread must call it).
template <int TPB>
__device__ __forceinline__ void block_partial(double v, double* partial, int slot) {
    __shared__ double ss[TPB], sc[TPB];
    ss[threadIdx.x] = v;
    sc[threadIdx.x] = 0.0;
    __syncthreads();
#pragma unroll
    for (int o = TPB / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            Comp a{ss[threadIdx.x], sc[threadIdx.x]}, b{ss[threadIdx.x + o], sc[threadIdx.x + o]};
            Comp c = comp_add(a, b);
            ss[threadIdx.x] = c.s;
            sc[threadIdx.x] = c.c;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) { partial[2 * slot] = ss[0]; partial[2 * slot + 1] = sc[0]; }
    __syncthreads();
}

// A warp-per-walker sweep's arrays and controls.  The standalone kernels fill
// one from their parameters, which ptxas re-reads at each use rather than
// holding registers across the sweep loop.  The batched kernels keep one per
// block in shared memory and pass it as volatile, so that each use is a
// shared load and, again, nothing is held in registers across the loop (a
// copy loaded once from the batch record in global memory would be).
template <class T>
struct SweepArgs {
    T* pos;
    T* dinv;
    int* sign;
    unsigned long long* acc;
    int* flags;
    uint64_t step0, seed;
    T step, tau, maxd;
    int W, Wcap, n_sweeps, fixed_node;
};

// A warp-per-walker refresh's arrays, block-shared for the same reason as
// SweepArgs (the kernels write the walker state at the end of a long walk).
template <class TS>
struct MeasureArgs {
    const TS* pos;
    TS* dinv;
    double* log;
    int* sign;
    double* el;
    double* grad;                  // optional per-electron outputs (null: not written)
    double* lap;
    int* flags;
    float2* rows;                  // two-launch refresh scratch (electron gas)
    const void* kt;                // reciprocal-space table (electron gas)
    int W, Wcap, write_state;
};

template <class TS>
__device__ __forceinline__ MeasureArgs<TS> measure_args(const BatchRec& R) {
    return MeasureArgs<TS>{(const TS*)R.pos, (TS*)R.dinv, R.logabs, R.sign, R.el, nullptr, nullptr, R.flags,
                           R.rows, R.ktab, R.W, R.Wcap, 1};
}

template <class T>
__device__ __forceinline__ SweepArgs<T> sweep_args(const BatchRec& R, const BatchCtl& c) {
    return SweepArgs<T>{(T*)R.pos, (T*)R.dinv, R.sign, R.acc, R.flags, c.step, batch_system_seed(c.seed, R.index),
                        (T)c.step_size, (T)c.tau, (T)c.max_drift, R.W, R.Wcap, c.n_sweeps, R.fixed_node};
}

// Persistent batched launches: block b owns the contiguous run of tiles
// [t0, t1) of the class's tile list, so consecutive tiles mostly share a
// system and its table is staged once per run.
__device__ __forceinline__ void batch_tile_range(int ntiles, int& t0, int& t1) {
    t0 = (int)(((long long)ntiles * blockIdx.x) / gridDim.x);
    t1 = (int)(((long long)ntiles * (blockIdx.x + 1)) / gridDim.x);
}

// Whole-block copy of a system table into shared memory (no barrier).
template <class TAB>
__device__ __forceinline__ void stage_table(TAB* dst, const void* src) {
    static_assert(sizeof(TAB) % 4 == 0, "table size must be a multiple of 4 bytes");
    const int* s = static_cast<const int*>(src);
    int* d = reinterpret_cast<int*>(dst);
    for (int i = threadIdx.x; i < (int)(sizeof(TAB) / 4); i += blockDim.x) d[i] = __ldg(s + i);
}

}  // namespace qmc

// Internal definitions shared by the SchwarMAX GB300 kernels.
//
// The canonical potential (likelihood.py:13-71) is evaluated inline with an
// analytic gradient.  For the Dehnen & Aly needle terms F_n (the needle
// convolution of M/r^n, dehnen_bar.py:104-157, 211-241) the gradient uses
//   dA_n/dx = Ax_n = R2^{-n/2},  dC_n/dx = A_n           (C_n = x A_n - B_n)
//   dF_n/du2 = -(n/2) F_{n+2}                            (d r^-n / d u2 = -(n/2) r^-(n+2))
// with u2 = y^2 + Z^2 and Z = sqrt(z^2 + b^2) + a, so one extra order of the
// value recurrence replaces a derivative recurrence.  The n = 1 terms use
// cancellation-free forms: A_1 = log(x + r) = log(u2 / (r - x)) for x < 0, and
// the needle difference A_1(x+L) - A_1(x-L) = log1p(2L (1 + 2|x|/(r+ + r-)) / D).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/schwarmax.h"

namespace smx {

constexpr double kG = 4.498502151469554e-06;          // kpc^3 / Msun / Gyr^2
constexpr double kKpcGyrToKms = 0.9777922216807892;
constexpr double kEps = 1e-12;                         // EPSILON of constants.py:11
constexpr double kPi = 3.14159265358979323846;

int set_error(int status, const char *fmt, ...);
// Process-wide count of kernels this library has launched (smx_kernel_launches).
void count_launch(unsigned n = 1);
int check_cuda(cudaError_t e, const char *what);
void clear_error();

#define SMX_TRY_CUDA(expr)                                              \
    do {                                                                \
        cudaError_t _e = (expr);                                        \
        if (_e != cudaSuccess) return ::smx::check_cuda(_e, #expr);     \
    } while (0)

// ---------------------------------------------------------------- math
template <typename T> struct M;
template <> struct M<float> {
    static __device__ __forceinline__ float rsqrt(float x) { return rsqrtf(x); }
    static __device__ __forceinline__ float sqrt(float x) { return sqrtf(x); }
    static __device__ __forceinline__ float log(float x) { return logf(x); }
    static __device__ __forceinline__ float log1p(float x) { return log1pf(x); }
    static __device__ __forceinline__ float rcbrt(float x) { return rcbrtf(x); }
    static __device__ __forceinline__ float exp(float x) { return expf(x); }
    static __device__ __forceinline__ float atan2(float y, float x) { return atan2f(y, x); }
    static __device__ __forceinline__ float asinh(float x) { return asinhf(x); }
    static __device__ __forceinline__ float abs(float x) { return fabsf(x); }
    // fast reciprocal (max 2 ulp) and square root of a positive argument (x rsqrt(x),
    // about 3 ulp): the exact forms cost several instructions each, and the force
    // evaluates about a dozen per call
    static __device__ __forceinline__ float rcp(float x) { return __fdividef(1.0f, x); }
    static __device__ __forceinline__ float sqrt_pos(float x) { return x * rsqrtf(x); }
};
template <> struct M<double> {
    static __device__ __forceinline__ double rsqrt(double x) { return ::rsqrt(x); }
    static __device__ __forceinline__ double sqrt(double x) { return ::sqrt(x); }
    static __device__ __forceinline__ double log(double x) { return ::log(x); }
    static __device__ __forceinline__ double log1p(double x) { return ::log1p(x); }
    static __device__ __forceinline__ double rcbrt(double x) { return ::rcbrt(x); }
    static __device__ __forceinline__ double exp(double x) { return ::exp(x); }
    static __device__ __forceinline__ double atan2(double y, double x) { return ::atan2(y, x); }
    static __device__ __forceinline__ double asinh(double x) { return ::asinh(x); }
    static __device__ __forceinline__ double abs(double x) { return ::fabs(x); }
    static __device__ __forceinline__ double rcp(double x) { return 1.0 / x; }
    static __device__ __forceinline__ double sqrt_pos(double x) { return ::sqrt(x); }
};

// ---------------------------------------------------------- reductions
// Fire-and-forget adds (red, relaxed, gpu scope) issued as inline PTX with no
// memory clobber, for scatter loops that keep per-sample arrays in local memory:
// there atomicAdd (global or shared) made the soft projection 19x slower (29.7 s
// against 1.55 s for the same 6.6e9 adds on 57.8M samples), while these leave the
// surrounding code as it is.  Nothing may read the target before the kernel ends.
static __device__ __forceinline__ void red_add(float *p, float v) {
    asm volatile("red.relaxed.gpu.global.add.f32 [%0], %1;" ::"l"(__cvta_generic_to_global(p)), "f"(v));
}
static __device__ __forceinline__ void red_add(double *p, double v) {
    asm volatile("red.relaxed.gpu.global.add.f64 [%0], %1;" ::"l"(__cvta_generic_to_global(p)), "d"(v));
}
static __device__ __forceinline__ void red_add(unsigned long long *p, unsigned long long v) {
    asm volatile("red.relaxed.gpu.global.add.u64 [%0], %1;" ::"l"(__cvta_generic_to_global(p)), "l"(v));
}

// -------------------------------------------------------- potential params
template <typename T> struct PotT {
    T GMh, iRs, iqa2, iqb2, iqc2;                 // NFW
    T GMd, Md, ad, bd2;                            // Miyamoto-Nagai
    T ba, ba3, bb2, bL, bc1, bc2;                  // T3 bar: c1 = M(1-g)/(2L), c2 = M g/L^2, ba3 = a/3
    T ua, ub2, uL, uc1, uc2;                       // V4 bulge
    T ua3;                                         // bulge a/3 (for a T3 in the bulge slot)
    int btype, utype;                              // Dehnen model of each slot (0: T3 / V4)
    int cyl_nr, cyl_nz, cyl_nm;                    // cylindrical-spline table (cyl_nm = 0: none)
    T cyl_r0;
    const double *cyl_r, *cyl_z, *cyl_c;
};

template <typename T> __host__ __device__ inline PotT<T> make_pot(const smx_potential &p) {
    PotT<T> q;
    q.GMh = T(kG * p.halo_M);
    q.iRs = T(1.0 / p.halo_Rs);
    q.iqa2 = T(1.0 / (p.halo_qa * p.halo_qa));
    q.iqb2 = T(1.0 / (p.halo_qb * p.halo_qb));
    q.iqc2 = T(1.0 / (p.halo_qc * p.halo_qc));
    q.GMd = T(kG * p.disc_M);
    q.Md = T(p.disc_M);
    q.ad = T(p.disc_a);
    q.bd2 = T(p.disc_b * p.disc_b);
    q.ba = T(p.bar_a);
    q.ba3 = T(p.bar_a / 3.0);
    q.bb2 = T(p.bar_b * p.bar_b);
    q.bL = T(p.bar_L);
    q.bc1 = T(p.bar_M * (1.0 - p.bar_gamma) / (2.0 * p.bar_L));
    q.bc2 = T(p.bar_M * p.bar_gamma / (p.bar_L * p.bar_L));
    q.ua = T(p.bulge_a);
    q.ub2 = T(p.bulge_b * p.bulge_b);
    q.uL = T(p.bulge_L);
    q.uc1 = T(p.bulge_M * (1.0 - p.bulge_gamma) / (2.0 * p.bulge_L));
    q.uc2 = T(p.bulge_M * p.bulge_gamma / (p.bulge_L * p.bulge_L));
    q.ua3 = T(p.bulge_a / 3.0);
    q.btype = p.bar_type == 0 ? 3 : p.bar_type;
    q.utype = p.bulge_type == 0 ? 14 : p.bulge_type;
    q.cyl_nm = p.cyl_n_modes > 0 ? p.cyl_n_modes : 0;
    q.cyl_nr = p.cyl_n_r;
    q.cyl_nz = p.cyl_n_z;
    q.cyl_r0 = T(p.cyl_n_modes > 0 ? p.cyl_r0 : 1.0);
    q.cyl_r = p.cyl_r_grid;
    q.cyl_z = p.cyl_z_grid;
    q.cyl_c = p.cyl_coef;
    return q;
}

int validate_potential(const smx_potential *p);

// ------------------------------------------------------------ needle sums
// Running state of the recurrence at one needle position xp: A_n, B_n and
// Ax_n = R2^{-n/2} at the current odd order n.
template <typename T> struct Rec {
    T xp, R2, iR2, r, A, B, Ax;
    __device__ __forceinline__ void init(T xp_, T u2) {
        xp = xp_;
        R2 = xp * xp + u2;
        const T ir = M<T>::rsqrt(R2);
        iR2 = ir * ir;
        r = R2 * ir;
        A = T(0);          // A_1 = log term is supplied separately when needed
        B = r;
        Ax = ir;
    }
    __device__ __forceinline__ T log_A1(T u2) const {
        return M<T>::log((xp >= T(0)) ? xp + r : u2 * M<T>::rcp(r - xp));
    }
    // advance n -> n + 2 (dehnen_bar.py:137-142)
    __device__ __forceinline__ void step(int n, T iu2) {
        const T inv_n = T(1) / T(n);
        const T An = ((T(n) - T(1)) * A + xp * Ax) * iu2 * inv_n;
        B = -Ax * inv_n;
        Ax = Ax * iR2;
        A = An;
    }
};

// Needle-convolved M/r^n (dehnen_bar.py:211-241, 269-278):
//   F_n = c1 [A_n(x+L) - A_n(x-L)] + c2 [C_n(x+L) + C_n(x-L) - 2 C_n(x)],  C_n = x A_n - B_n.
// Returns S0 = sum_k kc[k] F_{2k+1} and, with GRAD,
//   Sx = sum_k kc[k] dF/dx,  SZ = sum_k dkc[k] F,  Su = sum_k kc[k] dF/du2
// with dF_n/dx = c1 [Ax_n(+) - Ax_n(-)] + c2 [A_n(+) + A_n(-) - 2 A_n(0)] and, since F_n
// is the needle convolution of r^-n with r^2 = x^2 + u2,  dF_n/du2 = -(n/2) F_{n+2}
// (one order beyond the values is evaluated for it).  FIRST = first order index with
// a non-zero coefficient; orders below it are skipped, so the n = 1 logs are only
// evaluated when needed.
template <typename T, int K, int FIRST, bool GRAD>
__device__ __forceinline__ void needle_sum(T x, T u2, T L, T c1, T c2, const T (&kc)[K],
                                           const T (&dkc)[K], T &S0, T &Sx, T &Su, T &SZ) {
    const T iu2 = M<T>::rcp(u2);
    constexpr int KK = GRAD ? K + 1 : K;
    S0 = Sx = Su = SZ = T(0);
    if (c1 != T(0)) {
        Rec<T> p, m;
        p.init(x + L, u2);
        m.init(x - L, u2);
#pragma unroll
        for (int k = 0; k < KK; ++k) {
            if (k >= FIRST) {
                T F;
                if (k == 0) {
                    const T ax = M<T>::abs(x);
                    const T D = (x >= T(0)) ? (m.xp + m.r) : (p.r - p.xp);
                    F = c1 * M<T>::log1p(T(2) * L * (T(1) + T(2) * ax * M<T>::rcp(p.r + m.r)) * M<T>::rcp(D));
                } else {
                    F = c1 * (p.A - m.A);
                }
                if (k < K) {
                    S0 += kc[k] * F;
                    if (GRAD) {
                        Sx += kc[k] * (c1 * (p.Ax - m.Ax));
                        SZ += dkc[k] * F;
                    }
                }
                if (GRAD && k >= FIRST + 1) Su += kc[k - 1] * (T(-0.5) * T(2 * k - 1)) * F;
            }
            if (k + 1 < KK) {
                p.step(2 * k + 1, iu2);
                m.step(2 * k + 1, iu2);
            }
        }
    }
    if (c2 != T(0)) {
        Rec<T> p, m, o;
        p.init(x + L, u2);
        m.init(x - L, u2);
        o.init(x, u2);
        if (FIRST == 0) {
            p.A = p.log_A1(u2);
            m.A = m.log_A1(u2);
            o.A = o.log_A1(u2);
        }
#pragma unroll
        for (int k = 0; k < KK; ++k) {
            if (k >= FIRST) {
                const T Cp = p.xp * p.A - p.B, Cm = m.xp * m.A - m.B, Co = o.xp * o.A - o.B;
                const T F = c2 * (Cp + Cm - T(2) * Co);
                if (k < K) {
                    S0 += kc[k] * F;
                    if (GRAD) {
                        Sx += kc[k] * (c2 * (p.A + m.A - T(2) * o.A));
                        SZ += dkc[k] * F;
                    }
                }
                if (GRAD && k >= FIRST + 1) Su += kc[k - 1] * (T(-0.5) * T(2 * k - 1)) * F;
            }
            if (k + 1 < KK) {
                // (n-1) A_n vanishes at n = 1, so the log term never feeds n >= 3
                p.step(2 * k + 1, iu2);
                m.step(2 * k + 1, iu2);
                o.step(2 * k + 1, iu2);
            }
        }
    }
}

// ----------------------------------------------------- Dehnen-Aly models
// Potential (and gradient) of one Dehnen & Aly needle model, Phi = -G sum_k kc[k]
// F_{2k+1} with the coefficients of _make_explicit_fns (dehnen_bar.py:1272-1390):
// T1..T4 (types 1..4) and V1..V4 (11..14); dk = d kc / dZ with ze = Z - a.  a3 = a/3
// rounded once in double (the T3 coefficient a (Z - a/3)).
// FIXED != 0 selects the model at compile time (the canonical fast path of the
// integrator); FIXED == 0 dispatches on the run-time type.
template <typename T, bool WANT_PHI, bool WANT_GRAD, int FIXED = 0>
__device__ __forceinline__ void dehnen_phi(int type_rt, T a, T a3, T b2, T L, T c1, T c2, T x, T y, T z, T &phi, T &gx,
                                           T &gy, T &gz) {
    const int type = FIXED ? FIXED : type_rt;
    if (c1 == T(0) && c2 == T(0)) return;
    const T G = T(kG);
    const T ze = M<T>::sqrt_pos(z * z + b2);
    const T Z = ze + a;
    const T u2 = y * y + Z * Z;
    const T aZ = a * Z;
    const T iz = M<T>::rcp(ze);
    const T h = T(0.5) * b2;
    T S0 = T(0), Sx = T(0), Su = T(0), SZ = T(0);
    switch (type) {
        case 1: {   // T1 (dehnen_bar.py:1303-1307)
            const T kc[1] = {T(1)}, dk[1] = {T(0)};
            needle_sum<T, 1, 0, WANT_GRAD>(x, u2, L, c1, c2, kc, dk, S0, Sx, Su, SZ);
            break;
        }
        case 2: {   // T2 (1309-1316)
            const T kc[2] = {T(1), aZ}, dk[2] = {T(0), a};
            needle_sum<T, 2, 0, WANT_GRAD>(x, u2, L, c1, c2, kc, dk, S0, Sx, Su, SZ);
            break;
        }
        case 3: {   // T3 (1318-1326)
            const T kc[3] = {T(1), a * (Z - a3), aZ * aZ};
            const T dk[3] = {T(0), a, T(2) * a * aZ};
            needle_sum<T, 3, 0, WANT_GRAD>(x, u2, L, c1, c2, kc, dk, S0, Sx, Su, SZ);
            break;
        }
        case 4: {   // T4 (1328-1337)
            const T kc[4] = {T(1), a * (Z - T(0.4) * a), T(0.6) * a * aZ * (Z + Z - a), aZ * aZ * aZ};
            const T dk[4] = {T(0), a, T(0.6) * a * a * (T(4) * Z - a), T(3) * a * aZ * aZ};
            needle_sum<T, 4, 0, WANT_GRAD>(x, u2, L, c1, c2, kc, dk, S0, Sx, Su, SZ);
            break;
        }
        case 11: {  // V1 (1339-1346): d(Z/ze)/dZ = -a/ze^2
            const T kc[2] = {T(1), h * Z * iz}, dk[2] = {T(0), -h * a * iz * iz};
            needle_sum<T, 2, 0, WANT_GRAD>(x, u2, L, c1, c2, kc, dk, S0, Sx, Su, SZ);
            break;
        }
        case 12: {  // V2 (1348-1357): d(Z^2/ze)/dZ = Z (Z - 2a)/ze^2
            const T kc[3] = {T(1), aZ + h, T(3) * h * aZ * Z * iz};
            const T dk[3] = {T(0), a, T(3) * h * a * Z * (Z - a - a) * iz * iz};
            needle_sum<T, 3, 0, WANT_GRAD>(x, u2, L, c1, c2, kc, dk, S0, Sx, Su, SZ);
            break;
        }
        case 13: {  // V3 (1359-1369): d(Z^3/ze)/dZ = Z^2 (2Z - 3a)/ze^2
            const T kc[4] = {T(1), a * (Z - a3) + h, aZ * (aZ + T(3) * h), T(5) * h * aZ * aZ * Z * iz};
            const T dk[4] = {T(0), a, a * (T(2) * aZ + T(3) * h),
                             T(5) * h * a * a * Z * Z * (T(2) * Z - T(3) * a) * iz * iz};
            needle_sum<T, 4, 0, WANT_GRAD>(x, u2, L, c1, c2, kc, dk, S0, Sx, Su, SZ);
            break;
        }
        default: {  // 14: V4 (1371-1383)
            const T kc[5] = {T(1), a * (Z - T(0.4) * a) + h,
                             T(3) * a * (T(0.2) * aZ * (Z + Z - a) + h * (Z - T(0.2) * a)),
                             aZ * aZ * (aZ + T(6) * h), T(7) * h * aZ * aZ * aZ * Z * iz};
            const T dk[5] = {T(0), a, T(3) * a * (T(0.2) * a * (T(4) * Z - a) + h),
                             a * aZ * (T(3) * aZ + T(12) * h),
                             T(7) * h * aZ * aZ * aZ * (T(3) * Z - T(4) * a) * iz * iz};
            needle_sum<T, 5, 0, WANT_GRAD>(x, u2, L, c1, c2, kc, dk, S0, Sx, Su, SZ);
            break;
        }
    }
    if (WANT_PHI) phi += -G * S0;
    if (WANT_GRAD) {
        gx += -G * Sx;
        gy += -G * Su * T(2) * y;
        gz += -G * (SZ + Su * T(2) * Z) * (z * iz);
    }
}

// Density of one Dehnen & Aly model (dehnen_bar.py:1399-1543): (b^2 / ze^3) pref
// sum_k kd[k] F_{2k+1}, orders from the first non-zero coefficient.
template <typename T>
__device__ __forceinline__ T dehnen_rho(int type, T a, T b2, T L, T c1, T c2, T x, T y, T z) {
    if (c1 == T(0) && c2 == T(0)) return T(0);
    const T pi = T(kPi);
    const T ze = M<T>::sqrt(z * z + b2);
    const T iz = T(1) / ze;
    const T Z = ze + a;
    const T Z2 = Z * Z, A2 = a * a, AZ = a * Z;
    const T u2 = y * y + Z2;
    T S0 = T(0), Sx, Su, SZ;
    T pref;
    switch (type) {
        case 1: {
            const T kd[3] = {T(0), a, T(3) * Z2 * ze}, z0[3] = {T(0), T(0), T(0)};
            needle_sum<T, 3, 1, false>(x, u2, L, c1, c2, kd, z0, S0, Sx, Su, SZ);
            pref = T(0.25) / pi;
            break;
        }
        case 2: {
            const T kd[4] = {T(0), T(0), A2 * a + ze * ze * ze, T(5) * AZ * Z2 * ze}, z0[4] = {};
            needle_sum<T, 4, 2, false>(x, u2, L, c1, c2, kd, z0, S0, Sx, Su, SZ);
            pref = T(0.75) / pi;
            break;
        }
        case 3: {
            const T kd[5] = {T(0), T(0), T(3) * ze * ze * ze, T(5) * a * Z2 * ((T(3) * ze - T(2) * a) * ze + A2),
                             T(35) * A2 * Z2 * Z2 * ze};
            const T z0[5] = {};
            needle_sum<T, 5, 2, false>(x, u2, L, c1, c2, kd, z0, S0, Sx, Su, SZ);
            pref = T(0.25) / pi;
            break;
        }
        case 4: {
            const T ze3 = ze * ze * ze;
            const T kd[6] = {T(0), T(0), T(3) * ze3, T(15) * AZ * ze3, T(7) * A2 * Z * Z2 * ((T(6) * ze - T(3) * a) * ze + A2),
                             T(63) * A2 * AZ * Z2 * Z2 * ze};
            const T z0[6] = {};
            needle_sum<T, 6, 2, false>(x, u2, L, c1, c2, kd, z0, S0, Sx, Su, SZ);
            pref = T(0.25) / pi;
            break;
        }
        case 11: {
            const T kd[4] = {T(0), a * iz * iz, T(3) * AZ * iz, T(5) * Z * Z2}, z0[4] = {};
            needle_sum<T, 4, 1, false>(x, u2, L, c1, c2, kd, z0, S0, Sx, Su, SZ);
            pref = T(0.375) * b2 / pi;
            break;
        }
        case 12: {
            const T kd[5] = {T(0), T(0), T(3) * a * A2 * iz * iz, T(5) * Z2 * (ze * ze - T(2) * a * ze + T(3) * A2) * iz,
                             T(35) * a * Z2 * Z2};
            const T z0[5] = {};
            needle_sum<T, 5, 2, false>(x, u2, L, c1, c2, kd, z0, S0, Sx, Su, SZ);
            pref = T(0.375) * b2 / pi;
            break;
        }
        case 13: {
            const T ai = a * iz;
            const T kd[6] = {T(0), T(0), T(0), T(3) * ze * ze * ze * (T(1) + ai * ai * ai * ai * ai),
                             T(7) * AZ * Z2 * iz * ((T(3) * ze - T(4) * a) * ze + T(3) * A2), T(63) * A2 * Z * Z2 * Z2};
            const T z0[6] = {};
            needle_sum<T, 6, 3, false>(x, u2, L, c1, c2, kd, z0, S0, Sx, Su, SZ);
            pref = T(0.625) * b2 / pi;
            break;
        }
        default: {
            const T kd[7] = {T(0), T(0), T(0), T(5) * ze * ze * ze,
                             T(7) * a * Z2 * (T(5) * ze * ze - T(4) * a * ze + T(3) * A2 - T(2) * a * A2 * iz + A2 * A2 * iz * iz),
                             T(63) * A2 * Z2 * Z2 * (ze + ze - T(2) * a + A2 * iz),
                             T(231) * A2 * AZ * Z2 * Z2 * Z};
            const T z0[7] = {};
            needle_sum<T, 7, 3, false>(x, u2, L, c1, c2, kd, z0, S0, Sx, Su, SZ);
            pref = T(0.375) * b2 / pi;
            break;
        }
    }
    return (b2 * iz * iz * iz) * pref * S0;
}

// ------------------------------------------------------- cylindrical spline
// Interval of a sorted grid holding v: searchsorted(g, v) - 1 clipped to [0, n - 2]
// (CubicSpline.py:138-142), i.e. the first index with g >= v, minus one.
template <typename T>
__device__ __forceinline__ int grid_interval(const double *__restrict__ g, int n, T v) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (T(g[mid]) < v) lo = mid + 1;
        else hi = mid;
    }
    lo -= 1;
    return lo < 0 ? 0 : (lo > n - 2 ? n - 2 : lo);
}

// Phi and grad Phi of the cylindrical-spline expansion (CylindricalSpline.py:418-519):
// Phi = sum_m f_m (Re Phi_m(Rs, zs) cos m phi - Im Phi_m sin m phi), f_0 = 1, f_m = 2,
// with the separable bicubic of CubicSpline.py:202-305 on Rs = asinh(R/R0),
// zs = asinh(|z|/R0); nothing is added outside the grid (the reference's fill value 0).
// cos m phi and sin m phi come from x/R, y/R by the angle-addition recurrence.
template <typename T, bool WANT_PHI, bool WANT_GRAD>
__device__ __forceinline__ void cylspline(const PotT<T> &P, T x, T y, T z, T &phi, T &gx, T &gy, T &gz) {
    const int nr = P.cyl_nr, nz = P.cyl_nz;
    const T R = M<T>::sqrt(x * x + y * y), za = M<T>::abs(z), R0 = P.cyl_r0;
    const T Rs = M<T>::asinh(R / R0), zs = M<T>::asinh(za / R0);
    if (Rs < T(P.cyl_r[0]) || Rs > T(P.cyl_r[nr - 1]) || zs < T(P.cyl_z[0]) || zs > T(P.cyl_z[nz - 1])) return;
    const int ix = grid_interval<T>(P.cyl_r, nr, Rs), iy = grid_interval<T>(P.cyl_z, nz, zs);
    const T gx0 = T(P.cyl_r[ix]), hx = T(P.cyl_r[ix + 1]) - gx0;
    const T gy0 = T(P.cyl_z[iy]), hy = T(P.cyl_z[iy + 1]) - gy0;
    const T tx = (Rs - gx0) / hx, ty = (zs - gy0) / hy;
    const T ux = T(1) - tx, uy = T(1) - ty;
    const T cx = hx * hx / T(6), cy = hy * hy / T(6);
    const T wx0 = ux * ux * ux - ux, wx1 = tx * tx * tx - tx;      // value weights of M_x
    const T dx0 = T(-3) * ux * ux + T(1), dx1 = T(3) * tx * tx - T(1);
    const T wy0 = uy * uy * uy - uy, wy1 = ty * ty * ty - ty;
    const T dy0 = T(-3) * uy * uy + T(1), dy1 = T(3) * ty * ty - T(1);
    const bool rpos = R > T(1e-12);
    const T c1 = rpos ? x / R : T(1), s1 = rpos ? y / R : T(0);   // cos, sin of atan2(y, x)
    const int64_t plane = (int64_t)nr * nz;
    const int64_t k00 = (int64_t)ix * nz + iy;
    T S = T(0), dS_R = T(0), dS_z = T(0), dS_p = T(0);
    T cm = T(1), sm = T(0);
    for (int m = 0; m < P.cyl_nm; ++m) {
        const double *base = P.cyl_c + (int64_t)m * 6 * plane;
        T val[2], dvx[2], dvy[2];
#pragma unroll
        for (int part = 0; part < 2; ++part) {   // 0: real, 1: imaginary
            const double *v = base + part * plane, *Mx = base + (2 + 2 * part) * plane,
                         *My = base + (3 + 2 * part) * plane;
            const T z00 = T(v[k00]), z10 = T(v[k00 + nz]), z01 = T(v[k00 + 1]), z11 = T(v[k00 + nz + 1]);
            const T a00 = T(Mx[k00]), a10 = T(Mx[k00 + nz]), a01 = T(Mx[k00 + 1]), a11 = T(Mx[k00 + nz + 1]);
            const T b00 = T(My[k00]), b10 = T(My[k00 + nz]), b01 = T(My[k00 + 1]), b11 = T(My[k00 + nz + 1]);
            const T f0 = ux * z00 + tx * z10 + (wx0 * a00 + wx1 * a10) * cx;
            const T f1 = ux * z01 + tx * z11 + (wx0 * a01 + wx1 * a11) * cx;
            const T m0 = ux * b00 + tx * b10, m1 = ux * b01 + tx * b11;
            val[part] = uy * f0 + ty * f1 + (wy0 * m0 + wy1 * m1) * cy;
            if (WANT_GRAD) {
                const T df0 = (z10 - z00) + (dx0 * a00 + dx1 * a10) * cx;
                const T df1 = (z11 - z01) + (dx0 * a01 + dx1 * a11) * cx;
                dvx[part] = (uy * df0 + ty * df1 + (wy0 * (b10 - b00) + wy1 * (b11 - b01)) * cy) / hx;
                dvy[part] = ((f1 - f0) + (dy0 * m0 + dy1 * m1) * cy) / hy;
            }
        }
        const T f = m == 0 ? T(1) : T(2);
        S += f * (val[0] * cm - val[1] * sm);
        if (WANT_GRAD) {
            dS_R += f * (dvx[0] * cm - dvx[1] * sm);
            dS_z += f * (dvy[0] * cm - dvy[1] * sm);
            dS_p += f * (-T(m) * val[0] * sm - T(m) * val[1] * cm);
        }
        const T cn = cm * c1 - sm * s1;
        sm = sm * c1 + cm * s1;
        cm = cn;
    }
    if (WANT_PHI) phi += S;
    if (WANT_GRAD) {
        const T dphi_dR = dS_R / M<T>::sqrt(R * R + R0 * R0);
        const T sz = z > T(0) ? T(1) : (z < T(0) ? T(-1) : T(0));
        const T dphi_dz = dS_z / M<T>::sqrt(za * za + R0 * R0) * sz;
        if (rpos) {
            const T invR = T(1) / R;
            gx += dphi_dR * (x * invR) + dS_p * (-y * invR * invR);
            gy += dphi_dR * (y * invR) + dS_p * (x * invR * invR);
        }
        gz += dphi_dz;
    }
}

// ------------------------------------------------------------- potential
// Phi and/or its gradient (dPhi/dx, ...) of the canonical model at (x, y, z).
// CANON: the bar and bulge slots hold their default models (T3, V4), fixed at
// compile time; otherwise the slots' types are read from P.
template <typename T, bool WANT_PHI, bool WANT_GRAD, bool CANON = false>
__device__ __forceinline__ void potential(const PotT<T> &P, T x, T y, T z, T &phi, T &gx, T &gy, T &gz) {
    const T G = T(kG);
    const T eps = T(kEps);
    phi = gx = gy = gz = T(0);
    {   // NFW halo (potentials.py:18-27)
        const T s2 = x * x * P.iqa2 + y * y * P.iqb2 + z * z * P.iqc2 + eps;
        const T ir = M<T>::rsqrt(s2);
        const T r = s2 * ir;
        const T q = r * P.iRs;
        const T l = M<T>::log1p(q);
        const T ire = M<T>::rcp(r + eps);
        if (WANT_PHI) phi += -P.GMh * l * ire;
        if (WANT_GRAD) {
            const T dpdr = -P.GMh * (P.iRs * M<T>::rcp(T(1) + q) - l * ire) * ire;
            const T c = dpdr * ir;
            gx += c * x * P.iqa2;
            gy += c * y * P.iqb2;
            gz += c * z * P.iqc2;
        }
    }
    {   // Miyamoto-Nagai disc (potentials.py:51-65)
        const T rx = x + eps, ry = y + eps, rz = z + eps;
        const T zeta = M<T>::sqrt_pos(rz * rz + P.bd2);
        const T s = P.ad + zeta;
        const T iD = M<T>::rsqrt(rx * rx + ry * ry + s * s);
        if (WANT_PHI) phi += -P.GMd * iD;
        if (WANT_GRAD) {
            const T c = P.GMd * iD * iD * iD;
            gx += c * rx;
            gy += c * ry;
            gz += c * s * rz * M<T>::rcp(zeta);
        }
    }
    dehnen_phi<T, WANT_PHI, WANT_GRAD, CANON ? 3 : 0>(P.btype, P.ba, P.ba3, P.bb2, P.bL, P.bc1, P.bc2, x, y, z, phi,
                                                      gx, gy, gz);
    dehnen_phi<T, WANT_PHI, WANT_GRAD, CANON ? 14 : 0>(P.utype, P.ua, P.ua3, P.ub2, P.uL, P.uc1, P.uc2, x, y, z, phi,
                                                       gx, gy, gz);
    if (!CANON && P.cyl_nm > 0) cylspline<T, WANT_PHI, WANT_GRAD>(P, x, y, z, phi, gx, gy, gz);
}

// Stellar density MN + T3 + V4 (potentials.py:29-49, dehnen_bar.py:1425-1438, 1526-1543).
template <typename T>
__device__ __forceinline__ T density(const PotT<T> &P, T x, T y, T z) {
    const T eps = T(kEps);
    const T pi = T(kPi);
    T rho;
    {
        const T rx = x + eps, ry = y + eps, rz = z + eps;
        const T R2 = rx * rx + ry * ry;
        const T beta = M<T>::sqrt(rz * rz + P.bd2);
        const T ab = P.ad + beta;
        const T D2 = R2 + ab * ab;
        const T num = P.ad * R2 + (P.ad + T(3) * beta) * ab * ab;
        const T den = beta * beta * beta * D2 * D2 * M<T>::sqrt(D2);
        rho = (P.bd2 * P.Md / (T(4) * pi)) * (num / den);
    }
    rho += dehnen_rho<T>(P.btype, P.ba, P.bb2, P.bL, P.bc1, P.bc2, x, y, z);
    rho += dehnen_rho<T>(P.utype, P.ua, P.ub2, P.uL, P.uc1, P.uc2, x, y, z);
    return rho;
}

template <typename T, bool CANON = false>
__device__ __forceinline__ T phi_only(const PotT<T> &P, T x, T y, T z) {
    T p, a, b, c;
    potential<T, true, false, CANON>(P, x, y, z, p, a, b, c);
    return p;
}

// true when both Dehnen slots hold their default models
inline bool canonical_types(const smx_potential &p) {
    return (p.bar_type == 0 || p.bar_type == 3) && (p.bulge_type == 0 || p.bulge_type == 14) && p.cyl_n_modes == 0;
}

}  // namespace smx

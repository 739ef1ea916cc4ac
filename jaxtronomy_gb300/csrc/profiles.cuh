// Per-ray lens deflections and light profiles, templated on the arithmetic
// type.  The FP64 instantiation follows the reference formulas operation for
// operation; the FP32 instantiation uses constants precomputed in FP64 by the
// prepare kernel and forms that stay accurate in single precision.
//
// Reference formulas (JAXtronomy source tree):
//   SIE/NIE   LensModel/Profiles/nie.py:86-107,182-200,280-294 (sie.py:105-124)
//   EPL       LensModel/Profiles/epl.py:111-124,179-200,300-319,366-394,
//             Util/hyp2f1_util.py:135-176
//   SHEAR     LensModel/Profiles/shear.py:39-53
//   NFW       LensModel/Profiles/nfw.py:88-105,259-279,347-365,386-395
//   TNFW      LensModel/Profiles/tnfw.py:69-87,228-349
//   SERSIC    LensModel/Profiles/sersic_utils.py:69-110,239-267,
//             LightModel/Profiles/sersic_ellipse.py:62-93, sersic.py:54-73,
//             Util/param_util.py:103-123
#pragma once

#include "common.cuh"
#include "cse_table.h"

namespace lensgb {

// ---- record layouts (d[k] double, f[k+2] float for k >= 2) -----------------
// SIE/NIE : d2 b, d3 s, d4 q (clamped < 1), d5 cos phi, d6 sin phi,
//           d7 sqrt(1-q^2), d8 b/sqrt(1-q^2), d9 q^2, d10 q^2 s, d11 q^2 s^2
// EPL     : d2 b, d3 t, d4 q, d5 cos phi, d6 sin phi, d7 f, d8 nmax,
//           d9 2/(1+q) b^t
// SHEAR   : d2 gamma1, d3 gamma2
// NFW     : d2 Rs (floored), d3 rho0, d4 4 rho0 Rs, d5 1/Rs
// TNFW    : d2 Rs, d3 rho0, d4 tau, d5 4 rho0 Rs, d6 1/Rs, d7 1/tau,
//           d8 tau^2/(tau^2+1)^2, d9 tau^2 - 1, d10..d12 and d14..d25 the
//           bracket's polynomial outside x = max(tau, 1) (tnfw_far_f)
// SERSIC* : d2 amp, d3 R_sersic (floored), d4 1/R_sersic, d5 1/n, d6 b_n,
//           d7..d10 product-average transform (m00 m01 m10 m11)
constexpr int F_OFF = 2;  // float slot = double slot + F_OFF

template <typename R>
struct Rec {
    const R* v;  // points at slot 0 of the record in the working precision
    __device__ __forceinline__ R operator[](int k) const { return v[k]; }
};

// Slot of a type-specific value in the record of precision R.
template <typename R>
__device__ __forceinline__ int slot(int k) {
    return sizeof(R) == 8 ? k : k + F_OFF;
}

// ---------------------------------------------------------------------------
// NIE / SIE
// ---------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ void nie_deflect(const R* rec, R dx, R dy, R& ax, R& ay) {
    const R b = rec[slot<R>(2)], s = rec[slot<R>(3)], q = rec[slot<R>(4)];
    const R c = rec[slot<R>(5)], sn = rec[slot<R>(6)];
    const R sq = rec[slot<R>(7)], b_sq = rec[slot<R>(8)];
    const R q2s = rec[slot<R>(10)];
    (void)q;
    R x = dx * c + dy * sn;
    R y = -dx * sn + dy * c;
    R fx, fy;
    if (sizeof(R) == 8) {
        // psi = sqrt(q^2 (s^2 + x^2) + y^2), nie.py:339-345
        R psi = sqrt(q * q * (s * s + x * x) + y * y);
        fx = b_sq * atan(sq * x / (psi + s));
        fy = b_sq * atanh(sq * y / (psi + q2s));
    } else {
        const R q2 = rec[slot<R>(9)], q2s2 = rec[slot<R>(11)];
        R psi = sqrtf(fmaf(q2, x * x, fmaf(y, y, q2s2)));
        fx = b_sq * atanf(sq * x / (psi + s));
        fy = b_sq * atanhf(sq * y / (psi + q2s));
    }
    ax = fx * c - fy * sn;
    ay = fx * sn + fy * c;
}

// ---------------------------------------------------------------------------
// EPL (Tessore & Metcalf 2015 with the Lopez-Temme series of 2F1)
// ---------------------------------------------------------------------------
// F holds the nmax coefficients F_n of the series
//   2F1(1, t/2; 2 - t/2; z) = (1 - z/2)^-1 sum_n F_n w^n,  w = z / (z - 2)
// (hyp2f1_util.py:135-176 with a = 1, where the Pochhammer prefactor is 1).
// FP32 EPL.  With u = Z^2/|Z|^2 (|u| = 1) and z = -f u:
//   |z - 2|^2 = 4 |1 - z/2|^2 = 4 (1 + f u_r + f^2/4),
//   w = z/(z-2) = (f^2/4 + (f/2) u) / |1 - z/2|^2,
//   2F1 = S(w) (1 + (f/2) conj(u)) / |1 - z/2|^2,
// so one reciprocal serves both divisions, and (b/R)^t = b^t 2^(-t/2 log2 R^2)
// needs no square root.  Record: f4 b, f5 t, f6 q, f7 cos, f8 sin, f9 f,
// f10 nmax, f11 2/(1+q) b^t, f12 q cos, f13 q sin, f14 f^2/4, f15 f/2, f16 -t/2.
__device__ __forceinline__ void epl_deflect_f(const float* rec, const float* F, float dx, float dy,
                                              float& ax, float& ay) {
    const float c = rec[7], sn = rec[8], qc = rec[12], qs = rec[13];
    // FP32 series length (f17): the reference's nmax shortened to where the
    // remaining terms fall below FP32 resolution (set by the prepare kernel)
    const int nmax = (int)rec[17];
    const float pref = rec[11], f2q = rec[14], fh = rec[15], mth = rec[16];
    // Z = q x + i y in the profile frame
    const float za = fmaf(dx, qc, dy * qs), zb = fmaf(dy, c, -dx * sn);
    const float r2 = za * za + zb * zb;
    float hr = 1.f, hi = 0.f, ee = 1.f;
    if (nmax > 0) {
        if (r2 == 0.f) {  // reference: 0/0 at the centre -> NaN -> nan_to_num -> 0
            ax = 0.f;
            ay = 0.f;
            return;
        }
        // u only sets the phase of z (|u| = 1): a 2-ulp reciprocal suffices
        const float inv = __fdividef(1.f, r2);
        const float ur = (za * za - zb * zb) * inv, ui = 2.f * za * zb * inv;
        // 1/|1 - z/2|^2 by the hardware reciprocal (~1 ulp): measured on the
        // 1024-system EPL workload, the ray kernel 2.223 -> 2.141 ms with the
        // maximum FP32-vs-FP64 image error unchanged (5.69e-6)
        ee = __fdividef(1.f, fmaf(2.f * fh, ur, 1.f + f2q));
        const float wr = fmaf(fh, ur, f2q) * ee, wi = fh * ui * ee;
        // S(w) = sum_n F_n w^n with real F_n by division by the real quadratic
        // (x - w)(x - conj w) = x^2 - rr x - ss (Knuth, TAOCP 4.6.4):
        //   b_n = F_n + rr b_{n+1} + ss b_{n+2},  S(w) = (b_0 - wr b_1) + i wi b_1,
        // two real FMAs per term instead of a complex multiply-add's four; the
        // recurrence damps rounding errors by |w| <= f/(2 - f) < 1 per step.
        const float rr = 2.f * wr, ss = -fmaf(wr, wr, wi * wi);
        float b1 = F[nmax - 1], b2 = 0.f;  // b_{n+1}, b_{n+2}
        int n = nmax - 2;
        if ((nmax & 1) == 0) {  // odd number of remaining terms: one step first
            const float bn = fmaf(rr, b1, fmaf(ss, b2, F[n]));
            b2 = b1;
            b1 = bn;
            --n;
        }
        // two terms per trip, not unrolled further (same-box sweep of the ray
        // stage on the 1024-system workload: 1.684 ms, unrolled 2x 1.701, 3x
        // 1.829, 4x 1.775)
#pragma unroll 1
        for (; n >= 1; n -= 2) {
            // n is odd here, so (F[n-1], F[n]) is an aligned pair
            const float2 fp = *reinterpret_cast<const float2*>(F + n - 1);
            const float bn = fmaf(rr, b1, fmaf(ss, b2, fp.y));
            const float bm = fmaf(rr, bn, fmaf(ss, b1, fp.x));
            b2 = bn;
            b1 = bm;
        }
        const float sr = fmaf(-wr, b2, b1), si = wi * b2;
        // times (1 + (f/2) conj(u)) / |1 - z/2|^2
        const float gr = fmaf(fh, ur, 1.f), gi = -fh * ui;
        // (the factor 1/|1 - z/2|^2 goes into the amplitude below)
        hr = sr * gr - si * gi;
        hi = sr * gi + si * gr;
    }
    const float r2m = r2 > 1e-18f ? r2 : 1e-18f;  // R = max(|Z|, 1e-9)
    // hardware lg2/ex2: on the 1024-system EPL workload this moved the maximum
    // FP32 image error from 5.58e-6 to 5.69e-6 (rays it disturbs most are the
    // ones the FP64 refine pass recomputes)
    const float amp = (pref * ee) * ex2_approx(mth * lg2_approx(r2m));
    const float fx = amp * (za * hr - zb * hi);
    const float fy = amp * (za * hi + zb * hr);
    ax = fx * c - fy * sn;
    ay = fx * sn + fy * c;
}

// epl_deflect_f for NR rays of one profile at once (a row of a pixel's
// sub-rays): the same operations per ray, but one series loop for all NR
// (the trip count is the profile's), so the loop's control, moves and address
// arithmetic are shared and the rays' recurrences interleave.  A ray at Z = 0
// takes the same NaN-free zero as epl_deflect_f, by a select at the end.
template <int NR>
__device__ __forceinline__ void epl_deflect_f_row(const float* rec, const float* F,
                                                  const float* dx, const float* dy, float* ax,
                                                  float* ay) {
    const float c = rec[7], sn = rec[8], qc = rec[12], qs = rec[13];
    const int nmax = (int)rec[17];
    const float pref = rec[11], f2q = rec[14], fh = rec[15], mth = rec[16];
    float za[NR], zb[NR], r2[NR], hr[NR], hi[NR], ee[NR];
#pragma unroll
    for (int r = 0; r < NR; ++r) {
        za[r] = fmaf(dx[r], qc, dy[r] * qs);
        zb[r] = fmaf(dy[r], c, -dx[r] * sn);
        r2[r] = za[r] * za[r] + zb[r] * zb[r];
        hr[r] = 1.f;
        hi[r] = 0.f;
        ee[r] = 1.f;
    }
    if (nmax > 0) {
        float ur[NR], ui[NR], wr[NR], wi[NR], rr[NR], ss[NR], b1[NR], b2[NR];
#pragma unroll
        for (int r = 0; r < NR; ++r) {
            const float inv = __fdividef(1.f, r2[r]);
            ur[r] = (za[r] * za[r] - zb[r] * zb[r]) * inv;
            ui[r] = 2.f * za[r] * zb[r] * inv;
            ee[r] = __fdividef(1.f, fmaf(2.f * fh, ur[r], 1.f + f2q));
            wr[r] = fmaf(fh, ur[r], f2q) * ee[r];
            wi[r] = fh * ui[r] * ee[r];
            rr[r] = 2.f * wr[r];
            ss[r] = -fmaf(wr[r], wr[r], wi[r] * wi[r]);
            b1[r] = F[nmax - 1];
            b2[r] = 0.f;
        }
        int n = nmax - 2;
        if ((nmax & 1) == 0) {
#pragma unroll
            for (int r = 0; r < NR; ++r) {
                const float bn = fmaf(rr[r], b1[r], fmaf(ss[r], b2[r], F[n]));
                b2[r] = b1[r];
                b1[r] = bn;
            }
            --n;
        }
#pragma unroll 1
        for (; n >= 1; n -= 2) {
            const float2 fp = *reinterpret_cast<const float2*>(F + n - 1);
#pragma unroll
            for (int r = 0; r < NR; ++r) {
                const float bn = fmaf(rr[r], b1[r], fmaf(ss[r], b2[r], fp.y));
                const float bm = fmaf(rr[r], bn, fmaf(ss[r], b1[r], fp.x));
                b2[r] = bn;
                b1[r] = bm;
            }
        }
#pragma unroll
        for (int r = 0; r < NR; ++r) {
            const float sr = fmaf(-wr[r], b2[r], b1[r]), si = wi[r] * b2[r];
            const float gr = fmaf(fh, ur[r], 1.f), gi = -fh * ui[r];
            hr[r] = sr * gr - si * gi;
            hi[r] = sr * gi + si * gr;
        }
    }
#pragma unroll
    for (int r = 0; r < NR; ++r) {
        const float r2m = r2[r] > 1e-18f ? r2[r] : 1e-18f;
        const float amp = (pref * ee[r]) * ex2_approx(mth * lg2_approx(r2m));
        const float fx = amp * (za[r] * hr[r] - zb[r] * hi[r]);
        const float fy = amp * (za[r] * hi[r] + zb[r] * hr[r]);
        const bool zero = nmax > 0 && r2[r] == 0.f;  // reference: 0/0 -> NaN -> 0
        ax[r] = zero ? 0.f : fx * c - fy * sn;
        ay[r] = zero ? 0.f : fx * sn + fy * c;
    }
}

template <typename R>
__device__ __forceinline__ void epl_deflect(const R* rec, const R* F, R dx, R dy, R& ax, R& ay) {
    if (sizeof(R) == 4) {
        epl_deflect_f((const float*)rec, (const float*)F, (float)dx, (float)dy, (float&)ax,
                      (float&)ay);
        return;
    }
    // FP64: the reference's z = -f Z / conj(Z), w = z / (z - 2), 2F1 = S(w) / (1 - z/2)
    // and alpha = 2/(1+q) (b/R)^t Z 2F1 (epl.py:321-392, hyp2f1_util.py:135-176),
    // arranged for the FP64 pipe: one reciprocal serves |z - 2|^2 and
    // |1 - z/2|^2 = |z - 2|^2 / 4; the series S(w) = sum_n F_n w^n (real F_n) by
    // division by the real quadratic (x - w)(x - conj w) = x^2 - rr x - ss (two
    // FMAs per term instead of a complex multiply-add's four; |w| <= f/(2-f) < 1
    // damps its rounding); (b/R)^t = b^t exp(-t/2 ln max(|Z|^2, 1e-18)), i.e. the
    // reference's R = max(|Z|, 1e-9), without hypot or pow.
    const double t = rec[3], q = rec[4];
    const double c = rec[5], sn = rec[6], f = rec[7];
    const int nmax = (int)rec[8];
    const double pref = rec[9];
    const double x = dx * c + dy * sn;
    const double y = -dx * sn + dy * c;
    const double za = q * x, zb = y;  // Z = q x + i y
    const double r2 = za * za + zb * zb;
    double hr = 1, hi = 0;  // 2F1 value
    bool nan_case = false;
    if (nmax > 0) {
        if (r2 == 0.0) {
            nan_case = true;  // -f Z / conj(Z) is 0/0 at the centre -> NaN -> 0
        } else {
            const double inv = 1.0 / r2;
            const double zr = -f * (za * za - zb * zb) * inv;
            const double zi = -f * (2.0 * za * zb) * inv;
            const double dr = zr - 2.0, di = zi;
            const double dd = 1.0 / (dr * dr + di * di);
            const double wr = (zr * dr + zi * di) * dd;
            const double wi = (zi * dr - zr * di) * dd;
            const double rr = 2.0 * wr, ss = -(wr * wr + wi * wi);
            double b1 = F[nmax - 1], b2 = 0.0;  // b_{n+1}, b_{n+2}
            for (int n = nmax - 2; n >= 0; --n) {
                const double bn = fma(rr, b1, fma(ss, b2, F[n]));
                b2 = b1;
                b1 = bn;
            }
            const double sr = fma(-wr, b2, b1), si = wi * b2;
            const double er = 1.0 - 0.5 * zr, ei = -0.5 * zi;
            const double ee = 4.0 * dd;  // 1 / |1 - z/2|^2
            hr = (sr * er + si * ei) * ee;
            hi = (si * er - sr * ei) * ee;
        }
    }
    double fx, fy;
    if (nan_case) {
        fx = 0;
        fy = 0;
    } else {
        const double amp = pref * exp(-0.5 * t * log(r2 > 1e-18 ? r2 : 1e-18));
        const double omr = za * hr - zb * hi;
        const double omi = za * hi + zb * hr;
        fx = nan_to_num_1e10(amp * omr);
        fy = nan_to_num_1e10(amp * omi);
    }
    ax = (R)(fx * c - fy * sn);
    ay = (R)(fx * sn + fy * c);
}

// ---------------------------------------------------------------------------
// Circular multipoles m = 1, 3, 4 of EPL_MULTIPOLE_M1M3M4 (Xu et al. 2013, B12;
// multipole.py:72-119).  Record slots (double): d16 a1/2, d17 cos phi1,
// d18 sin phi1, d19 ln r_E, d20 a3/(1-9), d21 cos 3phi3, d22 sin 3phi3,
// d23 a4/(1-16), d24 cos 4phi4, d25 sin 4phi4, d26 phi1, d27 a3, d28 phi3,
// d29 a4, d30 phi4, d31 r_E = theta_E.
// ---------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ void multipole134_deflect(const R* rec, R dx, R dy, R& ax, R& ay) {
    if (sizeof(R) == 8) {
        // reference form: polar angle via atan2 (atan2(0, 0) = 0 at the centre)
        const double r0 = sqrt((double)dx * dx + (double)dy * dy);
        const double phi = atan2((double)dy, (double)dx);
        const double cph = cos(phi), sph = sin(phi);
        const double a1 = 2 * (double)rec[16], p1 = rec[26], rE = rec[31];
        const double r1 = r0 > 0.000001 ? r0 : 0.000001;
        const double lr = log(r1 / rE);
        double fx = a1 / 2 * (cos(p1) * lr + cos(phi - p1) * cph);
        double fy = a1 / 2 * (sin(p1) * lr + cos(phi - p1) * sph);
        const double am[2] = {rec[27], rec[29]}, pm[2] = {rec[28], rec[30]};
        const double mm[2] = {3.0, 4.0};
        for (int j = 0; j < 2; ++j) {
            const double m = mm[j], a = am[j], pj = pm[j];
            fx += cph * a / (1 - m * m) * cos(m * (phi - pj)) +
                  sph * m * a / (1 - m * m) * sin(m * (phi - pj));
            fy += sph * a / (1 - m * m) * cos(m * (phi - pj)) -
                  cph * m * a / (1 - m * m) * sin(m * (phi - pj));
        }
        ax = (R)fx;
        ay = (R)fy;
    } else {
        // FP32: cos/sin of the polar angle from the offsets, e^{i m phi} by powers
        const float* f = (const float*)rec;
        const float r2 = (float)dx * (float)dx + (float)dy * (float)dy;
        float c = 1.f, s = 0.f;
        if (r2 > 0.f) {
            const float ri = rsqrtf(r2);
            c = (float)dx * ri;
            s = (float)dy * ri;
        }
        const float r2m = r2 > 1e-12f ? r2 : 1e-12f;  // r floored at 1e-6
        const float lr = 0.5f * __logf(r2m) - f[21];
        const float cd1 = c * f[19] + s * f[20];      // cos(phi - phi1)
        float fx = f[18] * (f[19] * lr + cd1 * c);
        float fy = f[18] * (f[20] * lr + cd1 * s);
        const float C2 = c * c - s * s, S2 = 2.f * c * s;
        // m = 3
        const float C3 = C2 * c - S2 * s, S3 = S2 * c + C2 * s;
        const float cm3 = C3 * f[23] + S3 * f[24], sm3 = S3 * f[23] - C3 * f[24];
        fx += f[22] * (c * cm3 + 3.f * s * sm3);
        fy += f[22] * (s * cm3 - 3.f * c * sm3);
        // m = 4
        const float C4 = C2 * C2 - S2 * S2, S4 = 2.f * C2 * S2;
        const float cm4 = C4 * f[26] + S4 * f[27], sm4 = S4 * f[26] - C4 * f[27];
        fx += f[25] * (c * cm4 + 4.f * s * sm4);
        fy += f[25] * (s * cm4 - 4.f * c * sm4);
        ax = (R)fx;
        ay = (R)fy;
    }
}

// EPL_MULTIPOLE_M1M3M4 = EPL + the three multipoles about the same centre
// (epl_multipole_m1m3m4.py:608-678); the EPL part shares the EPL record layout.
template <typename R>
__device__ __forceinline__ void epl_multipole_deflect(const R* rec, const R* F, R dx, R dy, R& ax,
                                                      R& ay) {
    R ex, ey, mx, my;
    epl_deflect<R>(rec, F, dx, dy, ex, ey);
    multipole134_deflect<R>(rec, dx, dy, mx, my);
    ax = ex + mx;
    ay = ey + my;
}

// ---------------------------------------------------------------------------
// NFW_ELLIPSE_CSE: 44 cored steep ellipsoids (Oguri 2021), product-average
// coordinates (cored_steep_ellipsoid.py:227-245,434-477,536-564,
// nfw_ellipse_cse.py:250-280).  Record (double): d2 Rs, d3 1/Rs, d4 q, d5 cos,
// d6 sin, d7 sqrt(q), d9 4 rho0 Rs^2, d10 q^2, d11 1-q^2.  FP32 term table C:
// one float4 (q^2 s^2, s, q^2 s, a/s) per term.
// ---------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ void nfw_cse_deflect(const R* rec, const R* C, R dx, R dy, R& ax,
                                                R& ay);

template <>
__device__ __forceinline__ void nfw_cse_deflect<double>(const double* rec, const double* C,
                                                        double dx, double dy, double& ax,
                                                        double& ay) {
    const double Rs = rec[2], q = rec[4], c = rec[5], sn = rec[6];
    (void)C;
    double x = dx * c + dy * sn;
    double y = -dx * sn + dy * c;
    x = x / Rs;
    y = y / Rs;
    const double sq = sqrt(q);
    double fx = 0, fy = 0;
    for (int k = 0; k < CSE_NFW_TERMS; ++k) {
        const double a = kCseNfwA[k] / q, s = kCseNfwS[k];
        const double xa = x * sq, ya = y * sq;
        const double psi = sqrt(q * q * (s * s + xa * xa) + ya * ya);
        const double Phi = (psi + s) * (psi + s) + (1 - q * q) * xa * xa;
        const double gx = q * xa * (psi + q * q * s) / (s * psi * Phi);
        const double gy = q * ya * (psi + s) / (s * psi * Phi);
        fx += sq * (a * gx);
        fy += sq * (a * gy);
    }
    const double cst = rec[9];
    ax = cst * (fx * c - fy * sn);
    ay = cst * (fx * sn + fy * c);
}

template <>
__device__ __forceinline__ void nfw_cse_deflect<float>(const float* rec, const float* C, float dx,
                                                       float dy, float& ax, float& ay) {
    const float inv_rs = rec[5], c = rec[7], sn = rec[8], sq = rec[9];
    const float q2 = rec[12], omq2 = rec[13];
    const float x = (dx * c + dy * sn) * inv_rs * sq;  // product-average frame
    const float y = (-dx * sn + dy * c) * inv_rs * sq;
    const float B = q2 * x * x + y * y, D = omq2 * x * x;
    float sx = 0.f, sy = 0.f;
    const float4* T = reinterpret_cast<const float4*>(C);
#pragma unroll 4
    for (int k = 0; k < 44; ++k) {
        const float4 t = T[k];                    // (q^2 s^2, s, q^2 s, a/s)
        const float u = B + t.x;                  // psi^2 = q^2 (s^2 + x^2) + y^2
        const float psi = u * rsqrtf(u);
        const float ps = psi + t.y;
        const float Phi = fmaf(ps, ps, D);
        const float inv = __fdividef(t.w, psi * Phi);  // (a/s) / (psi Phi)
        sx = fmaf(psi + t.z, inv, sx);
        sy = fmaf(ps, inv, sy);
    }
    // sum_k a_k X (psi + q^2 s_k)/(s_k psi Phi), times sqrt(q) and the normalisation
    const float cst = rec[11] * sq;
    const float fx = cst * x * sx, fy = cst * y * sy;
    ax = fx * c - fy * sn;
    ay = fx * sn + fy * c;
}

// ---------------------------------------------------------------------------
// SHEAR
// ---------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ void shear_deflect(const R* rec, R dx, R dy, R& ax, R& ay) {
    const R g1 = rec[slot<R>(2)], g2 = rec[slot<R>(3)];
    ax = g1 * dx + g2 * dy;
    ay = g2 * dx - g1 * dy;
}

// CONVERGENCE (convergence.py:33-46): a mass sheet, alpha = kappa (x - ra_0).
// Record: d2 kappa, d3 kappa - fl(kappa) (the FP32 split's low part).
template <typename R>
__device__ __forceinline__ void convergence_deflect(const R* rec, R dx, R dy, R& ax, R& ay) {
    const R k = rec[slot<R>(2)];
    ax = k * dx;
    ay = k * dy;
}

// ---------------------------------------------------------------------------
// NFW
// ---------------------------------------------------------------------------
// G(X) = arccosh(1/X)/sqrt(1-X^2) (X<1), arccos(1/X)/sqrt(X^2-1) (X>1), 1 (X=1)
// is NFW's G and TNFW's F (tnfw.py:290-304).  FP32 evaluation:
//  * |1-X^2| < 0.12: the series sum_k w^k/(2k+1) with w = 1-X^2 (the quotient
//    of two vanishing numbers would lose all precision);
//  * X < 1: ln((1+u)/X)/u with u = sqrt(1-X^2) (= atanh(u)/u without the
//    1-u cancellation of atanh near 1);
//  * X > 1: atan(v)/v with v = sqrt(X^2-1).
__device__ __forceinline__ float nfw_G_f(float X) {
    float w = (1.f - X) * (1.f + X);
    if (fabsf(w) < 0.12f) {
        float s = 1.f / 23.f;
        s = fmaf(s, w, 1.f / 21.f);
        s = fmaf(s, w, 1.f / 19.f);
        s = fmaf(s, w, 1.f / 17.f);
        s = fmaf(s, w, 1.f / 15.f);
        s = fmaf(s, w, 1.f / 13.f);
        s = fmaf(s, w, 1.f / 11.f);
        s = fmaf(s, w, 1.f / 9.f);
        s = fmaf(s, w, 1.f / 7.f);
        s = fmaf(s, w, 1.f / 5.f);
        s = fmaf(s, w, 1.f / 3.f);
        return fmaf(s, w, 1.f);
    }
    if (w > 0.f) {
        float u = sqrtf(w);
        return logf((1.f + u) / X) / u;
    }
    float v = sqrtf(-w);
    return atanf(v) / v;
}

// g(X) = ln(X/2) + G(X) (nfw.py:347-365).  For X < 1 the two terms cancel to
// O(X^2 ln X); FP32 uses the equivalent cancellation-free form
//   g = [M X^2/(1+u) + log1p(-X^2/(2(1+u)))] / u,  M = ln(2/X), u = sqrt(1-X^2).
__device__ __forceinline__ float nfw_g_f(float X) {
    X = X < 0.000001f ? 0.000001f : X;
    float x2 = X * X;
    float w = (1.f - X) * (1.f + X);
    if (fabsf(w) < 0.12f) return logf(0.5f * X) + nfw_G_f(X);
    if (X < 1.f) {
        float u = sqrtf(w);
        float opu = 1.f + u;
        float M = logf(2.f / X);
        return (M * x2 / opu + log1pf(-x2 / (2.f * opu))) / u;
    }
    float v = sqrtf(-w);
    return logf(0.5f * X) + atanf(v) / v;
}

template <typename R>
__device__ __forceinline__ R nfw_g(R X) {
    if (sizeof(R) == 8) {
        X = X < R(0.000001) ? R(0.000001) : X;
        if (X < 1) return log(X / R(2)) + R(1) / sqrt(R(1) - X * X) * acosh(R(1) / X);
        if (X == 1) return R(1) + log(R(1) / R(2));
        return log(X / R(2)) + R(1) / sqrt(X * X - R(1)) * acos(R(1) / X);
    } else {
        return nfw_g_f(X);
    }
}

template <typename R>
__device__ __forceinline__ void nfw_deflect(const R* rec, R dx, R dy, R& ax, R& ay) {
    const R inv_rs = rec[slot<R>(5)], a4 = rec[slot<R>(4)];
    R Rr = sqrt(dx * dx + dy * dy);
    Rr = Rr > R(0.00000001) ? Rr : R(0.00000001);
    R X;
    if (sizeof(R) == 8)
        X = Rr / rec[slot<R>(2)];
    else
        X = Rr * inv_rs;
    R a = a4 * nfw_g<R>(X) / (X * X);
    ax = a * dx;
    ay = a * dy;
}

// ---------------------------------------------------------------------------
// TNFW
// ---------------------------------------------------------------------------
// The reference's powers w^-0.5, w^0.5 and w^-1 (tnfw.py:278-304) are taken
// as 1/sqrt(w), sqrt(w) and 1/w: the same values to an ulp, without pow.
__device__ __forceinline__ double tnfw_F_d(double x) {
    x = x > 0.001 ? x : 0.001;
    if (x < 1) {
        const double s = sqrt(1 - x * x);
        return atanh(s) / s;
    }
    if (x > 1) {
        const double s = sqrt(x * x - 1);
        return atan(s) / s;
    }
    return x;
}

// The bracket b(x) of g(x) = tau^2/(tau^2+1)^2 b(x) (tnfw.py:339-348).
__device__ __forceinline__ double tnfw_bracket_d(double x, double tau) {
    x = x > 0.001 ? x : 0.001;
    const double t2 = tau * tau;
    const double r = sqrt(t2 + x * x);
    const double L = log(x / (tau + r));
    return (t2 + 1 + 2 * (x * x - 1)) * tnfw_F_d(x) + tau * M_PI + (t2 - 1) * log(tau) +
           r * (-M_PI + L * (t2 - 1) / tau);
}

__device__ __forceinline__ double tnfw_g_d(double x, double tau) {
    const double t2 = tau * tau;
    return t2 / ((t2 + 1) * (t2 + 1)) * tnfw_bracket_d(x, tau);
}

// FP32 TNFW g.  The reference bracket (tnfw.py:339-348) cancels to O(x^2 ln x)
// for small x; regrouped exactly as
//   (t2-1) [x^2 L/(tau (tau+r)) - log1p(x^2/(2 tau (tau+r))) + g_NFW(x)]
//   + 2 x^2 F(x) - pi x^2/(tau+r),   r = sqrt(t2+x^2), L = ln(x/(tau+r)),
// every term of which is O(x^2 ln x) itself.
__device__ __forceinline__ float tnfw_g_f(float x, float tau) {
    x = x > 0.001f ? x : 0.001f;
    float t2 = tau * tau;
    float x2 = x * x;
    float r = sqrtf(t2 + x2);
    float tr = tau + r;
    float L = logf(x / tr);
    float B = x2 / (tau * tr) * L - log1pf(x2 / (2.f * tau * tr)) + nfw_g_f(x);
    float br = (t2 - 1.f) * B + 2.f * x2 * nfw_G_f(x) - 3.14159265358979f * x2 / tr;
    return t2 / ((t2 + 1.f) * (t2 + 1.f)) * br;
}

// FP32 TNFW deflection of one (ray, deflector) pair for many-deflector ray
// shooting: the same regrouped forms as tnfw_g_f / nfw_g_f / nfw_G_f with G(x)
// evaluated once, one reciprocal of tau + r shared by L and x^2/(tau (tau+r)),
// and the per-deflector constants of the record (f6 tau, f7 4 rho0 Rs,
// f8 1/Rs, f9 1/tau, f10 tau^2/(tau^2+1)^2, f11 tau^2 - 1).  Outside the
// truncation scale (x >= s = max(tau, 1): f12 holds s^2) the bracket b is the
// record's polynomial of degree TNFW_NC - 1 in t = 2 s/x - 1 (f16.., f14 = 2 s,
// f13 = 4 rho0 Rs tau^2/(tau^2+1)^2): b is analytic in z = s/x on the whole
// disk |z| < 1 (its nearest singularities are x = +-i tau), so its Chebyshev
// interpolant on z in [0, 1] converges geometrically -- 12 terms are within
// 1.3e-9 relative of b for tau in [0.05, 300] -- so the closed form, with its
// logarithms, is needed only inside x = s.
// The pair is split in two so that a thread's rays run the polynomial as
// straight-line code that interleaves: tnfw_far_f evaluates it whatever x and
// returns true when x < max(tau, 1), where the caller then overwrites the
// result with tnfw_near_f's closed form (a branch taken by ~1% of pairs).
// ESTRIN: the polynomial by Estrin's scheme (depth 4 instead of 11, two more
// multiplies) rather than Horner's.  The multi-plane kernel, whose 2-warp
// CTAs stall on dependent FMAs, gains; the single-plane bulk kernel, with more
// warps per SM, keeps Horner's.
template <bool ESTRIN = false>
__device__ __forceinline__ bool tnfw_far_f(const float* rec, float dx, float dy, float& ax,
                                           float& ay) {
    const float inv_rs = rec[8];
    const float u = fmaf(dx, dx, dy * dy) * (inv_rs * inv_rs);  // x^2
    {
        static_assert(TNFW_NC == 12, "three float4 loads of coefficients");
        const float e = rsqrtf(u);
        const float t = fmaf(rec[14], e, -1.f);
        const float4* cv = reinterpret_cast<const float4*>(rec + 16);
        const float4 q0 = cv[0], q1 = cv[1], q2 = cv[2];
        const float c[12] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w,
                             q2.x, q2.y, q2.z, q2.w};
        float b;
        if (ESTRIN) {
            const float t2 = t * t, t4 = t2 * t2, t8 = t4 * t4;
            float p[6];
#pragma unroll
            for (int k = 0; k < 6; ++k) p[k] = fmaf(c[2 * k + 1], t, c[2 * k]);
            const float e0 = fmaf(p[1], t2, p[0]), e1 = fmaf(p[3], t2, p[2]);
            const float e2 = fmaf(p[5], t2, p[4]);
            b = fmaf(e2, t8, fmaf(e1, t4, e0));
        } else {
            b = c[11];
#pragma unroll
            for (int k = 10; k >= 0; --k) b = fmaf(b, t, c[k]);
        }
        const float a = rec[13] * b * (e * e);
        ax = a * dx;
        ay = a * dy;
    }
    return !(u >= rec[12]);
}

__device__ __forceinline__ void tnfw_near_f(const float* rec, float dx, float dy, float& ax,
                                            float& ay) {
    const float tau = rec[6], a4 = rec[7], inv_rs = rec[8], inv_tau = rec[9];
    const float c0 = rec[10], tm1 = rec[11];
    const float t2 = tau * tau;
    // R >= 0.001 Rs and x >= 0.001 (tnfw.py:85, :335)
    float X = sqrtf(fmaf(dx, dx, dy * dy)) * inv_rs;
    X = X > 0.001f ? X : 0.001f;
    const float x2 = X * X;
    const float w = (1.f - X) * (1.f + X);
    float G, gn;
    if (fabsf(w) < 0.12f) {
        G = nfw_G_f(X);
        gn = logf(0.5f * X) + G;
    } else if (w > 0.f) {
        const float u = sqrtf(w);
        const float opu = 1.f + u;
        const float iu = __frcp_rn(u);
        G = logf(opu / X) * iu;
        gn = (logf(2.f / X) * x2 / opu + log1pf(-x2 / (2.f * opu))) * iu;
    } else {
        const float rv = rsqrtf(-w);
        G = atanf(-w * rv) * rv;
        gn = logf(0.5f * X) + G;
    }
    const float r = sqrtf(t2 + x2);
    const float itr = __frcp_rn(tau + r);
    const float L = logf(X * itr);
    const float p = x2 * itr * inv_tau;  // x^2 / (tau (tau + r))
    const float B = p * L - log1pf(0.5f * p) + gn;
    const float br = tm1 * B + 2.f * x2 * G - 3.14159265358979f * tau * p;
    const float a = a4 * (c0 * br) * __frcp_rn(x2);
    ax = a * dx;
    ay = a * dy;
}

template <typename R>
__device__ __forceinline__ void tnfw_deflect(const R* rec, R dx, R dy, R& ax, R& ay) {
    const R Rs = rec[slot<R>(2)], tau = rec[slot<R>(4)], a4 = rec[slot<R>(5)];
    R Rr = sqrt(dx * dx + dy * dy);
    Rr = Rr > R(0.001) * Rs ? Rr : R(0.001) * Rs;
    R X;
    R g;
    if (sizeof(R) == 8) {
        X = Rr / Rs;
        X = X > R(0.001) ? X : R(0.001);
        g = tnfw_g_d(X, tau);
    } else {
        X = Rr * rec[slot<R>(6)];
        X = X > R(0.001) ? X : R(0.001);
        g = tnfw_g_f(X, tau);
    }
    R a = a4 * g / (X * X);
    ax = a * dx;
    ay = a * dy;
}

// ---------------------------------------------------------------------------
// Sersic surface brightness (SERSIC and SERSIC_ELLIPSE share the record)
// ---------------------------------------------------------------------------
template <bool GRAD>
__device__ __forceinline__ float sersic_f(const float* rec, float dx, float dy, float& g);

template <typename R>
__device__ __forceinline__ R sersic_flux(const R* rec, R dx, R dy) {
    if (sizeof(R) == 4) {
        float g;
        return (R)sersic_f<false>((const float*)rec, (float)dx, (float)dy, g);
    }
    const R amp = rec[slot<R>(2)], inv_rs = rec[slot<R>(4)];
    const R inv_n = rec[slot<R>(5)], bn = rec[slot<R>(6)];
    const R m00 = rec[slot<R>(7)], m01 = rec[slot<R>(8)], m10 = rec[slot<R>(9)],
            m11 = rec[slot<R>(10)];
    R x = m00 * dx + m01 * dy;
    R y = m10 * dx + m11 * dy;
    R Rr = sqrt(x * x + y * y);
    R Rst = Rr > R(0.0001) ? Rr : R(0.0001);
    R frac;
    R res;
    if (sizeof(R) == 8) {
        frac = Rst / rec[3];
        R ex = -bn * (pow(frac, inv_n) - R(1));
        res = frac <= R(1000) ? exp(ex) : R(0);
    } else {
        frac = Rst * inv_rs;
        R ex = -bn * (exp2f(inv_n * log2f(frac)) - R(1));
        res = frac <= R(1000) ? expf(ex) : R(0);
    }
    return amp * nan_to_num_max(res);
}

// FP32 Sersic without a square root: with r2 = R^2 floored at 1e-8 (R floored
// at 1e-4),  log2(R/R_s) = log2(r2)/2 + log2(1/R_s),  v = (R/R_s)^(1/n),
// I = amp 2^(b_n log2(e) (1 - v)), zero beyond R/R_s = 1000.  With `grad`, also
// g = |d ln I / dR| = (b_n/n) v / R, the log-gradient that turns an absolute
// position error into a relative flux error (0 inside the smoothing floor).
// Record: f4 amp, f9..f12 transform, f13 log2(1/R_s), f14 b_n log2(e), f15 b_n/n.
template <bool GRAD>
__device__ __forceinline__ float sersic_f(const float* rec, float dx, float dy, float& g) {
    const float amp = rec[4], inv_n = rec[7];
    const float m00 = rec[9], m01 = rec[10], m10 = rec[11], m11 = rec[12];
    const float l2irs = rec[13], bnl = rec[14];
    const float x = m00 * dx + m01 * dy;
    const float y = m10 * dx + m11 * dy;
    const float r2 = x * x + y * y;
    const bool floored = !(r2 > 1e-8f);
    const float r2m = floored ? 1e-8f : r2;
    // log2(R/R_s): an absolute error of ~2^-22.6 here moves v by only ~4e-8/n
    const float l2f = fmaf(0.5f, lg2_approx(r2m), l2irs);
    // v is multiplied by b_n log2(e) (up to ~40) below; the hardware ex2 left the
    // maximum image error of the 1024-system EPL workload unchanged (5.58e-6)
    const float v = ex2_approx(inv_n * l2f);
    // the argument's own FP32 rounding dominates this exponential's error
    const float res = l2f <= 9.965784284662087f ? ex2_approx(bnl * (1.f - v)) : 0.f;
    if (GRAD) g = floored ? 0.f : rec[15] * v * rsqrtf(r2m);
    return amp * res;
}

__device__ __forceinline__ float sersic_flux_grad(const float* rec, float dx, float dy, float& g) {
    return sersic_f<true>(rec, dx, dy, g);
}

// ---------------------------------------------------------------------------
// Dispatch on the lens profile code (the name -> class table of
// LensModel/profile_list_base.py:309-765 for the profiles of this library).
// F is the profile's coefficient table (EPL series or CSE terms), if any.
// ---------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ void lens_deflect(int code, const R* rec, const R* F, R dx, R dy, R& ax,
                                             R& ay) {
    switch (code) {
        case LENSGB_LENS_SIE:
        case LENSGB_LENS_NIE: nie_deflect<R>(rec, dx, dy, ax, ay); break;
        case LENSGB_LENS_EPL: epl_deflect<R>(rec, F, dx, dy, ax, ay); break;
        case LENSGB_LENS_SHEAR: shear_deflect<R>(rec, dx, dy, ax, ay); break;
        case LENSGB_LENS_CONVERGENCE: convergence_deflect<R>(rec, dx, dy, ax, ay); break;
        case LENSGB_LENS_NFW: nfw_deflect<R>(rec, dx, dy, ax, ay); break;
        case LENSGB_LENS_TNFW: tnfw_deflect<R>(rec, dx, dy, ax, ay); break;
        case LENSGB_LENS_NFW_ELLIPSE_CSE: nfw_cse_deflect<R>(rec, F, dx, dy, ax, ay); break;
        case LENSGB_LENS_EPL_MULTIPOLE_M1M3M4:
            epl_multipole_deflect<R>(rec, F, dx, dy, ax, ay);
            break;
        default: ax = 0; ay = 0; break;
    }
}

// Deflections of NR rays by one profile of a compile-time stack: EPL by
// epl_deflect_f_row, any other profile ray by ray.
template <int NR>
__device__ __forceinline__ void lens_deflect_row_f(int code, const float* rec, const float* F,
                                                   const float* dx, const float* dy, float* ax,
                                                   float* ay) {
    if (code == LENSGB_LENS_EPL) {
        epl_deflect_f_row<NR>(rec, F, dx, dy, ax, ay);
        return;
    }
#pragma unroll
    for (int r = 0; r < NR; ++r) lens_deflect<float>(code, rec, F, dx[r], dy[r], ax[r], ay[r]);
}

}  // namespace lensgb

// Adjoint gradient of the image log-likelihood with respect to every
// parameter of every system row: d logL / d params, FP64.
//
// The reference differentiates ImageModel.likelihood_data_given_model with
// jax.grad (reverse mode through the XLA program, storing its intermediates;
// image_model.py:163-221, test_image_model.py:274-335).  Here the chain is
// written out and the ray grid is recomputed instead of stored:
//   1. logL and g_m = d logL / d m per pixel (residual weights of the
//      model-dependent variance  C = max(m,0)/t_exp + sigma_bkg^2 (+|err|) or
//      noise_map^2; imaging_data.py:159-182, image_noise.py:100-137);
//   2. the transpose of the image's numerics: the sub-frame crop
//      (numerics_subframe.py:87-149), the transposed "same"-mode convolution --
//      the convolution with the kernel rotated by 180 degrees, with zero
//      padding (PixelKernelConvolution, convolution.py:74-86) or through an
//      explicit edge-padded image whose halo is folded back onto the edge
//      pixels (GaussianConvolution, convolution.py:215-235) -- and for
//      convolution on the supersampled grid the transposed block mean and the
//      split kernel's pixel-scale part (SubgridKernelConvolution,
//      convolution.py:154-166), then the evaluation mask;
//   3. one thread per pixel recomputes its s^2 rays, forward-mode derivatives
//      of each lens deflection (EPL and EPL_MULTIPOLE_M1M3M4 through the
//      hypergeometric series with dF_n/dt tables, the multipoles analytically;
//      SIE/NIE; NFW/TNFW; the 44 CSE terms of NFW_ELLIPSE_CSE; CONVERGENCE;
//      SHEAR) and of each Sersic profile, and accumulates w * d flux / d p with
//      w = g_low * pixel_width^2 / s^2 * flux_scaling; the source terms reach
//      the lens parameters through
//      d beta / d p = -alpha_scaling * deflection_scaling * d alpha / d p;
//   4. per-CTA partial sums are reduced in a fixed order (deterministic).
// The EPL derivative uses the series of the forward pass (nmax(f) terms); the
// reference's custom JVP differentiates a 100-term series (epl.py:321-340),
// which differs from it by at most the series truncation (< 1e-10 relative).
#include "launch.h"
#include "profiles.cuh"
#include "raytrace_kernels.cuh"

namespace lensgb {

constexpr int GRAD_THREADS = 128;
constexpr int GRAD_PPT = 2;  // pixels per thread
constexpr int GJ = 12;       // parameters of the largest lens profile (EPL_MULTIPOLE_M1M3M4)

// ---------------------------------------------------------------------------
// forward-mode dual numbers with 5 tangent directions (b, t, q, x1, y1)
// ---------------------------------------------------------------------------
template <typename T>
struct D5 {
    T v;
    T d[5];
};

template <typename T>
__device__ __forceinline__ D5<T> dconst(T v) {
    D5<T> r;
    r.v = v;
#pragma unroll
    for (int k = 0; k < 5; ++k) r.d[k] = T(0.0);
    return r;
}
template <typename T>
__device__ __forceinline__ D5<T> dvar(T v, int k) {
    D5<T> r = dconst(v);
    r.d[k] = T(1.0);
    return r;
}
template <typename T>
__device__ __forceinline__ D5<T> operator+(const D5<T>& a, const D5<T>& b) {
    D5<T> r;
    r.v = a.v + b.v;
#pragma unroll
    for (int k = 0; k < 5; ++k) r.d[k] = a.d[k] + b.d[k];
    return r;
}
template <typename T>
__device__ __forceinline__ D5<T> operator-(const D5<T>& a, const D5<T>& b) {
    D5<T> r;
    r.v = a.v - b.v;
#pragma unroll
    for (int k = 0; k < 5; ++k) r.d[k] = a.d[k] - b.d[k];
    return r;
}
template <typename T>
__device__ __forceinline__ D5<T> operator*(const D5<T>& a, const D5<T>& b) {
    D5<T> r;
    r.v = a.v * b.v;
#pragma unroll
    for (int k = 0; k < 5; ++k) r.d[k] = a.v * b.d[k] + b.v * a.d[k];
    return r;
}
template <typename T>
__device__ __forceinline__ D5<T> operator*(T s, const D5<T>& a) {
    D5<T> r;
    r.v = s * a.v;
#pragma unroll
    for (int k = 0; k < 5; ++k) r.d[k] = s * a.d[k];
    return r;
}
template <typename T>
__device__ __forceinline__ D5<T> operator+(T s, const D5<T>& a) {
    D5<T> r = a;
    r.v += s;
    return r;
}
template <typename T>
__device__ __forceinline__ D5<T> dinv(const D5<T>& a) {
    D5<T> r;
    r.v = T(1.0) / a.v;
    const T g = -r.v * r.v;
#pragma unroll
    for (int k = 0; k < 5; ++k) r.d[k] = g * a.d[k];
    return r;
}
template <typename T>
__device__ __forceinline__ D5<T> dlog(const D5<T>& a) {
    D5<T> r;
    r.v = log(a.v);
    const T g = T(1.0) / a.v;
#pragma unroll
    for (int k = 0; k < 5; ++k) r.d[k] = g * a.d[k];
    return r;
}
template <typename T>
__device__ __forceinline__ D5<T> dexp(const D5<T>& a) {
    D5<T> r;
    r.v = exp(a.v);
#pragma unroll
    for (int k = 0; k < 5; ++k) r.d[k] = r.v * a.d[k];
    return r;
}
template <typename T>
__device__ __forceinline__ D5<T> dsqrt(const D5<T>& a) {
    D5<T> r;
    r.v = sqrt(a.v);
    const T g = T(0.5) / r.v;
#pragma unroll
    for (int k = 0; k < 5; ++k) r.d[k] = g * a.d[k];
    return r;
}
template <typename T>
__device__ __forceinline__ D5<T> datan(const D5<T>& a) {
    D5<T> r;
    r.v = atan(a.v);
    const T g = T(1.0) / (T(1.0) + a.v * a.v);
#pragma unroll
    for (int k = 0; k < 5; ++k) r.d[k] = g * a.d[k];
    return r;
}
template <typename T>
__device__ __forceinline__ D5<T> datanh(const D5<T>& a) {
    D5<T> r;
    r.v = atanh(a.v);
    const T g = T(1.0) / (T(1.0) - a.v * a.v);
#pragma unroll
    for (int k = 0; k < 5; ++k) r.d[k] = g * a.d[k];
    return r;
}

template <typename T>
__device__ __forceinline__ D5<T> dacosh(const D5<T>& a) {
    D5<T> r;
    r.v = acosh(a.v);
    const T g = T(1.0) / sqrt(a.v * a.v - T(1.0));
#pragma unroll
    for (int k = 0; k < 5; ++k) r.d[k] = g * a.d[k];
    return r;
}
template <typename T>
__device__ __forceinline__ D5<T> dacos(const D5<T>& a) {
    D5<T> r;
    r.v = acos(a.v);
    const T g = -T(1.0) / sqrt(T(1.0) - a.v * a.v);
#pragma unroll
    for (int k = 0; k < 5; ++k) r.d[k] = g * a.d[k];
    return r;
}

// (phi, q) = ellipticity2phi_q(e1, e2) (param_util.py:88-99): dq/de and dphi/de
// (zero at e = 0 and where the axis-ratio clamp c < 0.9999 holds it).
template <typename T>
__device__ __forceinline__ void dphiq_de(T e1, T e2, T& dq1, T& dq2,
                                         T& dp1, T& dp2) {
    const T cc2 = e1 * e1 + e2 * e2;
    const T cc = sqrt(cc2);
    dq1 = dq2 = dp1 = dp2 = T(0.0);
    if (cc > T(0.0)) {
        if (cc < T(0.9999)) {
            const T dqdc = -T(2.0) / ((T(1.0) + cc) * (T(1.0) + cc));
            dq1 = dqdc * e1 / cc;
            dq2 = dqdc * e2 / cc;
        }
        dp1 = -e2 / (T(2.0) * cc2);
        dp2 = e1 / (T(2.0) * cc2);
    }
}

// EPL deflection (epl.py:179-200,366-394) and its Jacobian with respect to
// (theta_E, gamma, e1, e2, center_x, center_y): J[0][k] = d alpha_x / d p_k,
// J[1][k] = d alpha_y / d p_k.  `a` is the profile's raw parameter row.
template <typename T>
__device__ void epl_alpha_grad(const T* rec, const T* F, const T* dF,
                               const T* a, T dx, T dy, T& ax, T& ay,
                               T J[2][GJ]) {
    const T b = rec[2], t = rec[3], q = rec[4], c = rec[5], sn = rec[6];
    const int nmax = (int)rec[8];
    const T x1 = c * dx + sn * dy, y1 = -sn * dx + c * dy;
    const D5<T> B = dvar(b, 0), Tt = dvar(t, 1), Q = dvar(q, 2);
    const D5<T> X1 = dvar(x1, 3), Y1 = dvar(y1, 4);
    const D5<T> Za = Q * X1, Zb = Y1;
    const D5<T> r2 = Za * Za + Zb * Zb;
    for (int i = 0; i < 2; ++i)
        for (int k = 0; k < GJ; ++k) J[i][k] = T(0.0);
    ax = T(0.0);
    ay = T(0.0);
    if (r2.v == T(0.0)) return;  // reference: 0/0 -> NaN -> nan_to_num -> 0
    D5<T> hr = dconst(T(1.0)), hi = dconst(T(0.0));
    if (nmax > 0) {
        const D5<T> f = (T(1.0) + (-T(1.0)) * Q) * dinv(T(1.0) + Q);
        const D5<T> inv = dinv(r2);
        const D5<T> zr = (-T(1.0)) * f * (Za * Za - Zb * Zb) * inv;
        const D5<T> zi = (-T(2.0)) * f * Za * Zb * inv;
        const D5<T> dr = zr + dconst(-T(2.0)), di = zi;
        const D5<T> dd = dinv(dr * dr + di * di);
        const D5<T> wr = (zr * dr + zi * di) * dd;
        const D5<T> wi = (zi * dr - zr * di) * dd;
        D5<T> sr = dconst(F[nmax - 1]);
        sr.d[1] = dF[nmax - 1];
        D5<T> si = dconst(T(0.0));
        for (int n = nmax - 2; n >= 0; --n) {
            D5<T> fn = dconst(F[n]);
            fn.d[1] = dF[n];
            const D5<T> nr = sr * wr - si * wi + fn;
            const D5<T> ni = sr * wi + si * wr;
            sr = nr;
            si = ni;
        }
        const D5<T> er = T(1.0) + (-T(0.5)) * zr, ei = (-T(0.5)) * zi;
        const D5<T> ee = dinv(er * er + ei * ei);
        hr = (sr * er + si * ei) * ee;
        hi = (si * er - sr * ei) * ee;
    }
    D5<T> R = dsqrt(r2);
    if (R.v < T(1e-9)) R = dconst(T(1e-9));
    // 2/(1+q) (b/R)^t
    const D5<T> amp = T(2.0) * dinv(T(1.0) + Q) * dexp(Tt * (dlog(B) - dlog(R)));
    const D5<T> fx = amp * (Za * hr - Zb * hi);
    const D5<T> fy = amp * (Za * hi + Zb * hr);
    ax = fx.v * c - fy.v * sn;
    ay = fx.v * sn + fy.v * c;
    // rotate the major-axis derivatives back
    T dA[2][5];
    for (int k = 0; k < 5; ++k) {
        dA[0][k] = fx.d[k] * c - fy.d[k] * sn;
        dA[1][k] = fx.d[k] * sn + fy.d[k] * c;
    }
    // d alpha / d phi = Rot(phi) [ (-fy, fx) + J_maj (y1, -x1) ]
    const T gx = -fy.v + fx.d[3] * y1 - fx.d[4] * x1;
    const T gy = fx.v + fy.d[3] * y1 - fy.d[4] * x1;
    const T aphx = gx * c - gy * sn, aphy = gx * sn + gy * c;
    // d alpha / d (dx, dy) = Rot(phi) J_maj Rot(-phi); (x1, y1) = Rot(-phi) (dx, dy)
    const T jdx0 = dA[0][3] * c - dA[0][4] * sn, jdx1 = dA[1][3] * c - dA[1][4] * sn;
    const T jdy0 = dA[0][3] * sn + dA[0][4] * c, jdy1 = dA[1][3] * sn + dA[1][4] * c;
    // chain to (theta_E, gamma, e1, e2): b = theta_E sqrt(q), t = gamma - 1,
    // (phi, q) from (e1, e2) (param_util.py:88-99, epl.py:111-124)
    const T theta_E = a[0], e1 = a[2], e2 = a[3];
    const T sq = sqrt(q);
    const T cc2 = e1 * e1 + e2 * e2;
    const T cc = sqrt(cc2);
    T dq1 = T(0.0), dq2 = T(0.0), dp1 = T(0.0), dp2 = T(0.0);
    if (cc > T(0.0)) {
        if (cc < T(0.9999)) {
            const T dqdc = -T(2.0) / ((T(1.0) + cc) * (T(1.0) + cc));
            dq1 = dqdc * e1 / cc;
            dq2 = dqdc * e2 / cc;
        }
        dp1 = -e2 / (T(2.0) * cc2);
        dp2 = e1 / (T(2.0) * cc2);
    }
    const T dbdq = theta_E / (T(2.0) * sq);
    for (int i = 0; i < 2; ++i) {
        const T aph = i == 0 ? aphx : aphy;
        const T aq = dA[i][0] * dbdq + dA[i][2];
        J[i][0] = dA[i][0] * sq;
        J[i][1] = dA[i][1];
        J[i][2] = aq * dq1 + aph * dp1;
        J[i][3] = aq * dq2 + aph * dp2;
        J[i][4] = -(i == 0 ? jdx0 : jdx1);
        J[i][5] = -(i == 0 ? jdy0 : jdy1);
    }
}

// NIE / SIE deflection (nie.py:86-107,182-200,280-294; sie.py:105-124 with
// s_scale = 1e-10) and its Jacobian with respect to (theta_E, e1, e2, [s_scale,]
// center_x, center_y).  b = theta_E sqrt(q) (the product-average conversion
// times sqrt((1 + q^2) / 2)), s = s_scale / sqrt(q); the major-axis formula is
// differentiated in (b, s, q, x1, y1), with q frozen where the q < 1 clamp
// replaces it.
template <typename T>
__device__ void nie_alpha_grad(int code, const T* rec, const T* a, T dx, T dy,
                               T& ax, T& ay, T J[2][GJ]) {
    const T b = rec[2], s = rec[3], qc = rec[4], c = rec[5], sn = rec[6];
    const bool nie = code == LENSGB_LENS_NIE;
    const T e1 = a[1], e2 = a[2];
    const T cc = sqrt(e1 * e1 + e2 * e2);
    const T q = (T(1.0) - fmin(cc, T(0.9999))) / (T(1.0) + fmin(cc, T(0.9999)));
    const bool clamped = q >= T(1.0);
    const T x1 = c * dx + sn * dy, y1 = -sn * dx + c * dy;
    const D5<T> B = dvar(b, 0), S = dvar(s, 1), Q = clamped ? dconst(qc) : dvar(qc, 2);
    const D5<T> X1 = dvar(x1, 3), Y1 = dvar(y1, 4);
    const D5<T> Q2 = Q * Q;
    const D5<T> psi = dsqrt(Q2 * (S * S + X1 * X1) + Y1 * Y1);
    const D5<T> sq = dsqrt(T(1.0) + (-T(1.0)) * Q2);
    const D5<T> bs = B * dinv(sq);
    const D5<T> fx = bs * datan(sq * X1 * dinv(psi + S));
    const D5<T> fy = bs * datanh(sq * Y1 * dinv(psi + Q2 * S));
    ax = fx.v * c - fy.v * sn;
    ay = fx.v * sn + fy.v * c;
    T dA[2][5];
    for (int k = 0; k < 5; ++k) {
        dA[0][k] = fx.d[k] * c - fy.d[k] * sn;
        dA[1][k] = fx.d[k] * sn + fy.d[k] * c;
    }
    // d alpha / d phi = Rot(phi) [ (-fy, fx) + J_maj (y1, -x1) ]
    const T gx = -fy.v + fx.d[3] * y1 - fx.d[4] * x1;
    const T gy = fx.v + fy.d[3] * y1 - fy.d[4] * x1;
    const T aphx = gx * c - gy * sn, aphy = gx * sn + gy * c;
    const T jdx0 = dA[0][3] * c - dA[0][4] * sn, jdx1 = dA[1][3] * c - dA[1][4] * sn;
    const T jdy0 = dA[0][3] * sn + dA[0][4] * c, jdy1 = dA[1][3] * sn + dA[1][4] * c;
    T dq1, dq2, dp1, dp2;
    dphiq_de(e1, e2, dq1, dq2, dp1, dp2);
    const T theta_E = a[0], s_scale = nie ? a[3] : T(0.0000000001);
    const T sqq = sqrt(q);
    const T dbdq = theta_E / (T(2.0) * sqq), dsdq = -s_scale / (T(2.0) * q * sqq);
    const int co = nie ? 4 : 3;
    for (int i = 0; i < 2; ++i) {
        const T aph = i == 0 ? aphx : aphy;
        const T aq = dA[i][0] * dbdq + dA[i][1] * dsdq + dA[i][2];
        J[i][0] = dA[i][0] * sqq;
        J[i][1] = aq * dq1 + aph * dp1;
        J[i][2] = aq * dq2 + aph * dp2;
        if (nie) J[i][3] = dA[i][1] / sqq;
        J[i][co] = -(i == 0 ? jdx0 : jdx1);
        J[i][co + 1] = -(i == 0 ? jdy0 : jdy1);
    }
}

// NFW (nfw.py:88-105, nfw_alpha :259-279, g :347-365, alpha2rho0 :386-395) and
// TNFW (tnfw.py:69-87, tnfw_alpha :228-248, _g :331-349, F :290-304, _L :278-286)
// deflections and their Jacobians with respect to (Rs, alpha_Rs, [r_trunc,]
// center_x, center_y), as dual numbers in (Rs, alpha_Rs, r_trunc, x, y) through
// the same formulas and floors as the forward pass (a floor freezes its
// argument's derivative).
template <typename T>
__device__ void nfw_alpha_grad(int code, const T* a, T dx, T dy, T& ax,
                               T& ay, T J[2][GJ]) {
    const bool trunc = code == LENSGB_LENS_TNFW;
    const D5<T> RS = dvar(a[0], 0), ARS = dvar(a[1], 1);
    const D5<T> X1 = dvar(dx, 3), Y1 = dvar(dy, 4);
    // rho0 from the unfloored Rs, as alpha2rho0 does (nfw.py:386-395)
    const D5<T> rho0 = ARS * dinv((T(4.0) * (T(1.0) + log(T(0.5)))) * (RS * RS));
    D5<T> R = dsqrt(X1 * X1 + Y1 * Y1);
    D5<T> g, X, RSF;
    if (!trunc) {
        RSF = a[0] < T(0.0000001) ? dconst(T(0.0000001)) : RS;
        if (!(R.v > T(0.00000001))) R = dconst(T(0.00000001));
        X = R * dinv(RSF);
        if (X.v < T(0.000001)) X = dconst(T(0.000001));
        if (X.v < T(1.0))
            g = dlog(T(0.5) * X) + dinv(dsqrt(T(1.0) + (-T(1.0)) * X * X)) * dacosh(dinv(X));
        else if (X.v == T(1.0))
            g = dconst(T(1.0) + log(T(0.5)));
        else
            g = dlog(T(0.5) * X) + dinv(dsqrt(X * X + dconst(-T(1.0)))) * dacos(dinv(X));
    } else {
        RSF = RS;
        const D5<T> tau = dvar(a[2], 2) * dinv(RS);
        if (!(R.v > T(0.001) * a[0])) R = T(0.001) * RS;
        X = R * dinv(RS);
        if (!(X.v > T(0.001))) X = dconst(T(0.001));
        const D5<T> x2 = X * X;
        D5<T> F;
        if (X.v < T(1.0)) {
            const D5<T> w = dsqrt(T(1.0) + (-T(1.0)) * x2);
            F = dinv(w) * datanh(w);
        } else if (X.v > T(1.0)) {
            const D5<T> w = dsqrt(x2 + dconst(-T(1.0)));
            F = dinv(w) * datan(w);
        } else {
            F = X;
        }
        const D5<T> t2 = tau * tau;
        const D5<T> r = dsqrt(t2 + x2);
        const D5<T> L = dlog(X * dinv(tau + r));
        const D5<T> tp1 = t2 + dconst(T(1.0)), tm1 = t2 + dconst(-T(1.0));
        const D5<T> br = (tp1 + T(2.0) * (x2 + dconst(-T(1.0)))) * F + T(M_PI) * tau + tm1 * dlog(tau) +
                      r * (dconst(-T(M_PI)) + L * tm1 * dinv(tau));
        g = t2 * dinv(tp1 * tp1) * br;
    }
    const D5<T> al = T(4.0) * rho0 * RSF * g * dinv(X * X);
    const D5<T> fx = al * X1, fy = al * Y1;
    ax = fx.v;
    ay = fy.v;
    const int co = trunc ? 3 : 2;
    for (int i = 0; i < 2; ++i) {
        const D5<T>& f = i == 0 ? fx : fy;
        J[i][0] = f.d[0];
        J[i][1] = f.d[1];
        if (trunc) J[i][2] = f.d[2];
        J[i][co] = -f.d[3];
        J[i][co + 1] = -f.d[4];
    }
}

// SHEAR (shear.py:39-53) and its Jacobian w.r.t. (gamma1, gamma2, ra_0, dec_0).
template <typename T>
__device__ __forceinline__ void shear_alpha_grad(const T* rec, T dx, T dy,
                                                 T& ax, T& ay, T J[2][GJ]) {
    const T g1 = rec[2], g2 = rec[3];
    ax = g1 * dx + g2 * dy;
    ay = g2 * dx - g1 * dy;
    J[0][0] = dx;  J[1][0] = -dy;
    J[0][1] = dy;  J[1][1] = dx;
    J[0][2] = -g1; J[1][2] = -g2;
    J[0][3] = -g2; J[1][3] = g1;
    J[0][4] = J[0][5] = J[1][4] = J[1][5] = T(0.0);
}

// CONVERGENCE (convergence.py:35-46): alpha = kappa (x - ra_0, y - dec_0), and
// its Jacobian w.r.t. (kappa, ra_0, dec_0).
template <typename T>
__device__ __forceinline__ void convergence_alpha_grad(const T* rec, T dx, T dy,
                                                       T& ax, T& ay, T J[2][GJ]) {
    const T k = rec[2];
    ax = k * dx;
    ay = k * dy;
    J[0][0] = dx;  J[1][0] = dy;
    J[0][1] = -k;  J[1][1] = T(0.0);
    J[0][2] = T(0.0); J[1][2] = -k;
}

// NFW_ELLIPSE_CSE (nfw_ellipse_cse.py:250-280 -> cored_steep_ellipsoid.py:
// 227-245,434-477,536-564) and its Jacobian w.r.t. (Rs, alpha_Rs, e1, e2,
// center_x, center_y): the 44-term CSE sum in the product-average frame as dual
// numbers in (Rs, alpha_Rs, q, x1, y1), with the normalisation
// 4 rho0 Rs^3 / Rs = alpha_Rs / (1 + ln 1/2) (nfw.py:386-395), rotated back and
// chained to (e1, e2) through (phi, q) as for EPL.
template <typename T>
__device__ void cse_alpha_grad(const T* rec, const T* a, T dx, T dy,
                               T& ax, T& ay, T J[2][GJ]) {
    const T q = rec[4], c = rec[5], sn = rec[6];
    const T x1 = c * dx + sn * dy, y1 = -sn * dx + c * dy;
    const D5<T> RS = dvar(a[0], 0), ARS = dvar(a[1], 1), Q = dvar(q, 2);
    const D5<T> X1 = dvar(x1, 3), Y1 = dvar(y1, 4);
    const D5<T> iRS = dinv(RS);
    const D5<T> sq = dsqrt(Q);
    const D5<T> xa = X1 * iRS * sq, ya = Y1 * iRS * sq;
    const D5<T> q2 = Q * Q, omq2 = T(1.0) + (-T(1.0)) * q2;
    const D5<T> xa2 = xa * xa, ya2 = ya * ya;
    const D5<T> iq = dinv(Q);
    D5<T> fx = dconst(T(0.0)), fy = dconst(T(0.0));
    for (int k = 0; k < CSE_NFW_TERMS; ++k) {
        const T s = T(kCseNfwS[k]);
        const D5<T> am = T(kCseNfwA[k]) * iq;
        const D5<T> psi = dsqrt(q2 * (xa2 + dconst(s * s)) + ya2);
        const D5<T> ps = psi + dconst(s);
        const D5<T> Phi = ps * ps + omq2 * xa2;
        const D5<T> den = dinv(s * (psi * Phi));
        fx = fx + am * (Q * xa * (psi + s * q2) * den);
        fy = fy + am * (Q * ya * ps * den);
    }
    const D5<T> cst = (T(1.0) / (T(1.0) + log(T(0.5)))) * ARS * sq;
    fx = cst * fx;
    fy = cst * fy;
    ax = fx.v * c - fy.v * sn;
    ay = fx.v * sn + fy.v * c;
    T dA[2][5];
    for (int k = 0; k < 5; ++k) {
        dA[0][k] = fx.d[k] * c - fy.d[k] * sn;
        dA[1][k] = fx.d[k] * sn + fy.d[k] * c;
    }
    const T gx = -fy.v + fx.d[3] * y1 - fx.d[4] * x1;
    const T gy = fx.v + fy.d[3] * y1 - fy.d[4] * x1;
    const T aphx = gx * c - gy * sn, aphy = gx * sn + gy * c;
    const T jdx0 = dA[0][3] * c - dA[0][4] * sn, jdx1 = dA[1][3] * c - dA[1][4] * sn;
    const T jdy0 = dA[0][3] * sn + dA[0][4] * c, jdy1 = dA[1][3] * sn + dA[1][4] * c;
    T dq1, dq2, dp1, dp2;
    dphiq_de(a[2], a[3], dq1, dq2, dp1, dp2);
    for (int i = 0; i < 2; ++i) {
        const T aph = i == 0 ? aphx : aphy;
        J[i][0] = dA[i][0];
        J[i][1] = dA[i][1];
        J[i][2] = dA[i][2] * dq1 + aph * dp1;
        J[i][3] = dA[i][2] * dq2 + aph * dp2;
        J[i][4] = -(i == 0 ? jdx0 : jdx1);
        J[i][5] = -(i == 0 ? jdy0 : jdy1);
    }
}

// EPL_MULTIPOLE_M1M3M4 (epl_multipole_m1m3m4.py:463-535,608-678): the EPL part
// (epl_alpha_grad on the shared record) plus the multipoles m = 1, 3, 4 of
// multipole.py:72-119 with a_m = a{m}_a theta_E / sqrt(q), phi_m = phi +
// delta_phi_m and r_E = theta_E.  Jacobian w.r.t. (theta_E, gamma, e1, e2,
// center_x, center_y, a1_a, delta_phi_m1, a3_a, delta_phi_m3, a4_a,
// delta_phi_m4).  The multipoles are linear in a_m; their position derivatives
// go through the polar radius (m = 1 only, zero where r is floored at 1e-6)
// and the polar angle (zero at the centre itself, where atan2 has none).
template <typename T>
__device__ void multipole_alpha_grad(const T* rec, const T* F, const T* dF,
                                     const T* a, T dx, T dy, T& ax,
                                     T& ay, T J[2][GJ]) {
    epl_alpha_grad(rec, F, dF, a, dx, dy, ax, ay, J);
    const T q = rec[4], rE = rec[31];
    const T r0 = sqrt(dx * dx + dy * dy);
    const T phi = atan2(dy, dx);
    const T cph = cos(phi), sph = sin(phi);
    const T r1 = r0 > T(0.000001) ? r0 : T(0.000001);
    const T L = log(r1 / rE);
    const T am[3] = {T(2.0) * rec[16], rec[27], rec[29]};
    const T pm[3] = {rec[26], rec[28], rec[30]};
    T fx = T(0.0), fy = T(0.0);
    T dfa[3][2], dfp[3][2];    // d f / d a_m, d f / d phi_m
    T dfr[2] = {T(0.0), T(0.0)};     // d f / d r (through ln r, m = 1)
    T dfph[2] = {T(0.0), T(0.0)};    // d f / d (polar angle)
    T dfrE[2];                 // d f / d r_E
    {
        const T A = am[0], P = pm[0];
        const T cp = cos(P), sp = sin(P), cd = cos(phi - P), sd = sin(phi - P);
        const T ux = T(0.5) * (cp * L + cd * cph), uy = T(0.5) * (sp * L + cd * sph);
        fx += A * ux;
        fy += A * uy;
        dfa[0][0] = ux;
        dfa[0][1] = uy;
        dfp[0][0] = T(0.5) * A * (-sp * L + sd * cph);
        dfp[0][1] = T(0.5) * A * (cp * L + sd * sph);
        dfrE[0] = -T(0.5) * A * cp / rE;
        dfrE[1] = -T(0.5) * A * sp / rE;
        if (r0 > T(0.000001)) {
            dfr[0] += T(0.5) * A * cp / r0;
            dfr[1] += T(0.5) * A * sp / r0;
        }
        // d/dphi of cos(phi - P) cos(phi) and cos(phi - P) sin(phi)
        dfph[0] += T(0.5) * A * (-sd * cph - cd * sph);
        dfph[1] += T(0.5) * A * (-sd * sph + cd * cph);
    }
    for (int j = 1; j < 3; ++j) {
        const T m = j == 1 ? T(3.0) : T(4.0), A = am[j], P = pm[j];
        const T k = T(1.0) / (T(1.0) - m * m);
        const T C = cos(m * (phi - P)), S = sin(m * (phi - P));
        const T ux = k * (cph * C + m * sph * S), uy = k * (sph * C - m * cph * S);
        fx += A * ux;
        fy += A * uy;
        dfa[j][0] = ux;
        dfa[j][1] = uy;
        dfp[j][0] = A * k * m * (cph * S - m * sph * C);
        dfp[j][1] = A * k * m * (sph * S + m * cph * C);
        dfph[0] += -A * sph * C;
        dfph[1] += A * cph * C;
    }
    ax += fx;
    ay += fy;
    // position: d/d(dx, dy) = d/dr (cos, sin) + d/dphi (-sin, cos) / r
    T fdx[2], fdy[2];
    const T ir = r0 > T(0.0) ? T(1.0) / r0 : T(0.0);
    for (int i = 0; i < 2; ++i) {
        fdx[i] = dfr[i] * cph - dfph[i] * sph * ir;
        fdy[i] = dfr[i] * sph + dfph[i] * cph * ir;
    }
    const T theta_E = a[0], sqq = sqrt(q);
    T dq1, dq2, dp1, dp2;
    dphiq_de(a[2], a[3], dq1, dq2, dp1, dp2);
    for (int i = 0; i < 2; ++i) {
        T dth = dfrE[i], dq = T(0.0), dphi_epl = T(0.0);
        for (int j = 0; j < 3; ++j) {
            const T araw = a[6 + 2 * j];
            dth += dfa[j][i] * araw / sqq;
            dq += dfa[j][i] * (-T(0.5) * am[j] / q);
            dphi_epl += dfp[j][i];
            J[i][6 + 2 * j] = dfa[j][i] * theta_E / sqq;
            J[i][7 + 2 * j] = dfp[j][i];
        }
        J[i][0] += dth;
        J[i][2] += dq * dq1 + dphi_epl * dp1;
        J[i][3] += dq * dq2 + dphi_epl * dp2;
        J[i][4] -= i == 0 ? fdx[0] : fdx[1];
        J[i][5] -= i == 0 ? fdy[0] : fdy[1];
    }
}

// Sersic / elliptical Sersic (sersic_ellipse.py:62-93, sersic_utils.py:69-110,
// 239-267) at offset (dx, dy): value, gradient with respect to the offset,
// and derivatives with respect to the raw parameters (amp, R_sersic, n_sersic,
// [e1, e2,] center_x, center_y).
template <typename T>
__device__ void sersic_grad(int code, const T* rec, const T* a, T dx, T dy,
                            T& I, T& gx, T& gy, T dI[7]) {
    const bool ell = code == LENSGB_LIGHT_SERSIC_ELLIPSE;
    const int np = ell ? 7 : 5;
    for (int k = 0; k < np; ++k) dI[k] = T(0.0);
    I = T(0.0);
    gx = T(0.0);
    gy = T(0.0);
    const T amp = rec[2], Rs = rec[3], inv_n = rec[5], bn = rec[6];
    const T m00 = rec[7], m01 = rec[8], m10 = rec[9], m11 = rec[10];
    const T xp = m00 * dx + m01 * dy, yp = m10 * dx + m11 * dy;
    const T Rraw = sqrt(xp * xp + yp * yp);
    const bool floored = !(Rraw > T(0.0001));
    const T R = floored ? T(0.0001) : Rraw;
    const T frac = R / Rs;
    if (!(frac <= T(1000.0))) return;
    const T v = pow(frac, inv_n);
    const T res = exp(-bn * (v - T(1.0)));
    I = amp * res;
    // d ln I / d R (zero inside the smoothing floor)
    const T dlR = floored ? T(0.0) : -bn * inv_n * v / R;
    T dRdx = T(0.0), dRdy = T(0.0);
    if (!floored) {
        dRdx = (xp * m00 + yp * m10) / R;
        dRdy = (xp * m01 + yp * m11) / R;
    }
    gx = I * dlR * dRdx;
    gy = I * dlR * dRdy;
    const T n = a[2];
    dI[0] = res;                                                  // amp
    dI[1] = a[1] > T(0.0001) ? I * bn * inv_n * v / Rs : T(0.0);        // R_sersic (floors)
    const T dbn = (T(1.9992) * n - T(0.3271)) > T(0.00001) ? T(1.9992) : T(0.0);
    dI[2] = I * (-dbn * (v - T(1.0)) + bn * v * log(frac) * inv_n * inv_n);  // n_sersic
    int k = 3;
    if (ell) {
        const T e1 = a[3], e2 = a[4];
        const T n2 = T(1.0) - e1 * e1 - e2 * e2;
        const T nrm_raw = sqrt(fabs(n2));
        const bool nfl = !(nrm_raw > T(0.000001));
        const T nrm = nfl ? T(0.000001) : nrm_raw;
        const T sgn = n2 > 0 ? -T(1.0) : T(1.0);
        const T dn1 = nfl ? T(0.0) : sgn * e1 / nrm, dn2 = nfl ? T(0.0) : sgn * e2 / nrm;
        // x' = ((1-e1) dx - e2 dy)/norm, y' = (-e2 dx + (1+e1) dy)/norm
        const T dxp1 = -dx / nrm - xp * dn1 / nrm, dyp1 = dy / nrm - yp * dn1 / nrm;
        const T dxp2 = -dy / nrm - xp * dn2 / nrm, dyp2 = -dx / nrm - yp * dn2 / nrm;
        if (!floored) {
            dI[3] = I * dlR * (xp * dxp1 + yp * dyp1) / R;
            dI[4] = I * dlR * (xp * dxp2 + yp * dyp2) / R;
        }
        k = 5;
    }
    dI[k] = -gx;      // center_x
    dI[k + 1] = -gy;  // center_y
}

constexpr int GRAD_MAXP = 64;
constexpr int GRAD_MAX_LENSP = 32;

__device__ __host__ __forceinline__ int lens_np(int code) {
    switch (code) {
        case LENSGB_LENS_EPL: return 6;
        case LENSGB_LENS_NIE: return 6;
        case LENSGB_LENS_SIE: return 5;
        case LENSGB_LENS_SHEAR: return 4;
        case LENSGB_LENS_NFW: return 4;
        case LENSGB_LENS_TNFW: return 5;
        case LENSGB_LENS_CONVERGENCE: return 3;
        case LENSGB_LENS_NFW_ELLIPSE_CSE: return 6;
        case LENSGB_LENS_EPL_MULTIPOLE_M1M3M4: return 12;
        default: return 0;
    }
}

// dF_n/dt of the EPL series coefficients (hyp2f1_util.py:156-166 with
// B = t/2, C = 2 - t/2), one thread per (system, EPL profile).
__global__ void epl_dcoef_kernel(StackDesc st, int n_inst, const double* __restrict__ rec_d,
                                 const double* __restrict__ coef_d, double* __restrict__ dcoef) {
    const int gid = blockIdx.x * blockDim.x + threadIdx.x;
    const int n_prof = st.n_lens + st.n_src + st.n_ll;
    if (gid >= n_inst * st.n_lens) return;
    const int inst = gid / st.n_lens, p = gid % st.n_lens;
    const int es = st.epl_slot[p];
    if (es < 0 || (st.lens[p] != LENSGB_LENS_EPL && st.lens[p] != LENSGB_LENS_EPL_MULTIPOLE_M1M3M4))
        return;
    const double* d = rec_d + ((long long)inst * n_prof + p) * REC_D;
    const double* F = coef_d + ((long long)inst * st.n_epl + es) * EPL_NMAX;
    double* dF = dcoef + ((long long)inst * st.n_epl + es) * EPL_NMAX;
    const int nmax = (int)d[8];
    const double t = d[3], Bc = t / 2.0, C = 2.0 - Bc, K = 2.0 * Bc - C;
    if (nmax > 0) dF[0] = 0.0;
    if (nmax > 1) dF[1] = -2.0 / (C * C);
    for (int n = 2; n < nmax; ++n)
        dF[n] = ((n - 1.0) * dF[n - 2] - 1.5 * F[n - 1] - K * dF[n - 1] + 0.5 * F[n]) /
                (C + n - 1.0);
}

// logL (same Kahan order as loglike_kernel) and g_m = d logL / d m.
__global__ void __launch_bounds__(256)
loglike_weights_kernel(const double* __restrict__ model, long long npix, LoglikeArgs a,
                       double* __restrict__ gm, double* __restrict__ out) {
    const int inst = blockIdx.x;
    const double* m = model + (long long)inst * npix;
    const double* d = a.data + (long long)inst * a.data_stride;
    const double* nm = a.noise_map ? a.noise_map + (long long)inst * a.noise_stride : nullptr;
    const double* ex = a.exposure ? a.exposure + (long long)inst * a.exposure_stride : nullptr;
    const double* mask = a.mask ? a.mask + (long long)inst * a.mask_stride : nullptr;
    double* g = gm + (long long)inst * npix;
    const double b2 = a.background_rms * a.background_rms;
    double sum = 0.0, comp = 0.0;
    for (long long i = threadIdx.x; i < npix; i += 256) {
        const double mk = mask ? mask[i] : 1.0;
        if (mk == 0.0) {
            g[i] = 0.0;
            continue;
        }
        const double mv = m[i];
        double c, dc = 0.0;
        if (nm) {
            c = nm[i] * nm[i];
        } else {
            const double e = ex ? ex[i] : a.exposure_time;
            c = (mv >= 0 ? mv : 0.0) / e + b2;
            dc = mv > 0 ? 1.0 / e : 0.0;
        }
        if (a.error_map) c += fabs(a.error_map[i]);
        const double r = mv - d[i];
        const double term = r * r / c * mk;
        const double y = term - comp;
        const double t = sum + y;
        comp = (t - sum) - y;
        sum = t;
        // logL = -1/2 sum mask r^2 / C(m)
        g[i] = -mk * (r / c - 0.5 * r * r * dc / (c * c));
    }
    __shared__ double red[256];
    red[threadIdx.x] = sum;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[inst] = -red[0] / 2.0;
}

// PSF rotated by 180 degrees (the kernel of the transposed convolution).
__global__ void flip_psf_kernel(const double* __restrict__ in, double* __restrict__ out, int K,
                                long long in_stride, int n) {
    const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long kk = (long long)K * K;
    if (gid >= kk * n) return;
    const long long inst = gid / kk, j = gid % kk;
    out[inst * kk + j] = in[inst * in_stride + (kk - 1 - j)];
}

// Step 3: per-CTA partial gradients of one system.  T = double: every ray
// derivative in FP64.  T = float (FP32 split): the records, EPL tables and the
// parameter row are copied to FP32 once per CTA; each pixel's offsets of its
// first ray from every profile centre are formed in FP64 and rounded once,
// the sub-ray displacements (below a pixel) are added in FP32, the dual numbers
// run in FP32, and each thread's sums go to the FP64 block reduction.
//
// Pixels whose FP32 derivatives would be ill-conditioned -- rays landing near a
// steep source centre, where beta = theta - alpha cancels and FP32's few-ulp
// error of alpha moves d I / d beta by (|grad ln I| + 1/R) kappa |alpha| in
// relative terms -- are flagged (FLAG_PASS: flag[pix] = 1, the pixel's FP32
// terms dropped) and recomputed by the FP64 instantiation over the flagged
// pixels only (ONLY_FLAGGED), into a second set of partial sums.
constexpr int GRAD_ALL = 0, GRAD_FLAG_PASS = 1, GRAD_ONLY_FLAGGED = 2;
constexpr float GRAD_KAPPA = 3e-7f;  // FP32 relative error bound of a deflection

template <typename T>
__global__ void __launch_bounds__(GRAD_THREADS)
grad_ray_kernel(GridDesc g, StackDesc st, const double* __restrict__ params,
                const double* __restrict__ rec, const double* __restrict__ coef,
                const double* __restrict__ dcoef, const double* __restrict__ glow,
                double w_scale, double* __restrict__ partial, unsigned char* __restrict__ flag,
                float tau, int mode) {
    constexpr bool F32 = sizeof(T) == 4;
    extern __shared__ double smem[];
    const int inst = blockIdx.y;
    const int n_prof = st.n_lens + st.n_src + st.n_ll;
    const int NP = st.n_params;
    double* srec = smem;
    double* scoef = srec + n_prof * REC_D;
    double* sdcoef = scoef + st.n_epl * EPL_NMAX;
    load_records<double>(st, rec, coef, inst, srec, scoef);
    for (int p = 0; p < st.n_lens; ++p) {
        const int es = st.epl_slot[p];
        if (es < 0) continue;
        const int nmax = (int)srec[p * REC_D + 8];
        const double* gc = dcoef + ((long long)inst * st.n_epl + es) * EPL_NMAX;
        for (int k = threadIdx.x; k < nmax; k += blockDim.x) sdcoef[es * EPL_NMAX + k] = gc[k];
    }
    __syncthreads();
    const double* Pd = params + (long long)inst * NP;
    const T* trec = reinterpret_cast<const T*>(srec);
    const T* tcoef = reinterpret_cast<const T*>(scoef);
    const T* tdcoef = reinterpret_cast<const T*>(sdcoef);
    const T* P = reinterpret_cast<const T*>(Pd);
    if (F32) {
        // FP32 copies after the FP64 arrays
        float* f = reinterpret_cast<float*>(sdcoef + st.n_epl * EPL_NMAX);
        const int nr = n_prof * REC_D, nc = st.n_epl * EPL_NMAX;
        for (int k = threadIdx.x; k < nr; k += blockDim.x) f[k] = (float)srec[k];
        for (int k = threadIdx.x; k < nc; k += blockDim.x) {
            f[nr + k] = (float)scoef[k];
            f[nr + nc + k] = (float)sdcoef[k];
        }
        for (int k = threadIdx.x; k < NP; k += blockDim.x) f[nr + 2 * nc + k] = (float)Pd[k];
        __syncthreads();
        trec = reinterpret_cast<const T*>(f);
        tcoef = reinterpret_cast<const T*>(f + nr);
        tdcoef = reinterpret_cast<const T*>(f + nr + nc);
        P = reinterpret_cast<const T*>(f + nr + 2 * nc);
    }
    T acc[GRAD_MAXP], pacc[GRAD_MAXP];
    for (int k = 0; k < NP; ++k) acc[k] = T(0);
    const long long npix = (long long)g.nx * g.ny;
    const long long base = (long long)blockIdx.x * GRAD_THREADS * GRAD_PPT;
    const double* gl = glow + (long long)inst * npix;
    const double inv_s2 = 1.0 / ((double)g.s * g.s);
    const T alpha_scaling = (T)st.alpha_scaling;
    const T axf = (T)g.ax, bxf = (T)g.bx, ayf = (T)g.ay, byf = (T)g.by;
    for (int kk = 0; kk < GRAD_PPT; ++kk) {
        const long long pix = base + (long long)kk * GRAD_THREADS + threadIdx.x;
        if (pix >= npix) break;
        const int row = (int)(pix / g.nx), col = (int)(pix % g.nx);
        const double wd = gl[pix] * w_scale * inv_s2 * st.flux_scaling;
        if (wd == 0.0) continue;
        if (mode == GRAD_ONLY_FLAGGED && !flag[(long long)inst * npix + pix]) continue;
        const T w = (T)wd;
        // this pixel's terms, kept apart until its rays are known well-conditioned
        T* tgt = mode == GRAD_FLAG_PASS ? pacc : acc;
        if (mode == GRAD_FLAG_PASS)
            for (int k = 0; k < NP; ++k) pacc[k] = T(0);
        bool ill = false;
        // FP32: the first ray's offsets from every profile centre, in FP64, rounded once
        T ox[MAX_PROF * 3], oy[MAX_PROF * 3];
        if (F32) {
            const double X0 = g.ra00 + (double)(col * g.s) * g.ax + (double)(row * g.s) * g.bx;
            const double Y0 = g.dec00 + (double)(col * g.s) * g.ay + (double)(row * g.s) * g.by;
            for (int p = 0; p < n_prof; ++p) {
                ox[p] = (T)(X0 - srec[p * REC_D + RD_CX]);
                oy[p] = (T)(Y0 - srec[p * REC_D + RD_CY]);
            }
        }
        for (int si = 0; si < g.s; ++si) {
            for (int sj = 0; sj < g.s; ++sj) {
                const int I = row * g.s + si, Jc = col * g.s + sj;
                double X = 0.0, Y = 0.0;
                T ddx_s = T(0), ddy_s = T(0);
                if (F32) {
                    ddx_s = (T)sj * axf + (T)si * bxf;
                    ddy_s = (T)sj * ayf + (T)si * byf;
                } else {
                    X = g.ra00 + (double)Jc * g.ax + (double)I * g.bx;
                    Y = g.dec00 + (double)Jc * g.ay + (double)I * g.by;
                }
                // offset of this ray from the centre of profile p
                auto off = [&](int p, T& dx, T& dy) {
                    if (F32) {
                        dx = ox[p] + ddx_s;
                        dy = oy[p] + ddy_s;
                    } else {
                        dx = (T)(X - srec[p * REC_D + RD_CX]);
                        dy = (T)(Y - srec[p * REC_D + RD_CY]);
                    }
                };
                T axs = T(0), ays = T(0);
                T dA[2][GRAD_MAX_LENSP];
                int lp = 0;
                for (int p = 0; p < st.n_lens; ++p) {
                    const T* r = trec + p * REC_D;
                    const int code = st.lens[p];
                    const int es = st.epl_slot[p];
                    T ax, ay, J[2][GJ];
                    T ddx, ddy;
                    off(p, ddx, ddy);
                    if (code == LENSGB_LENS_EPL)
                        epl_alpha_grad(r, tcoef + es * EPL_NMAX, tdcoef + es * EPL_NMAX,
                                       P + st.lens_off[p], ddx, ddy, ax, ay, J);
                    else if (code == LENSGB_LENS_EPL_MULTIPOLE_M1M3M4)
                        multipole_alpha_grad(r, tcoef + es * EPL_NMAX, tdcoef + es * EPL_NMAX,
                                             P + st.lens_off[p], ddx, ddy, ax, ay, J);
                    else if (code == LENSGB_LENS_SIE || code == LENSGB_LENS_NIE)
                        nie_alpha_grad(code, r, P + st.lens_off[p], ddx, ddy, ax, ay, J);
                    else if (code == LENSGB_LENS_NFW || code == LENSGB_LENS_TNFW)
                        nfw_alpha_grad(code, P + st.lens_off[p], ddx, ddy, ax, ay, J);
                    else if (code == LENSGB_LENS_NFW_ELLIPSE_CSE)
                        cse_alpha_grad(r, P + st.lens_off[p], ddx, ddy, ax, ay, J);
                    else if (code == LENSGB_LENS_CONVERGENCE)
                        convergence_alpha_grad(r, ddx, ddy, ax, ay, J);
                    else
                        shear_alpha_grad(r, ddx, ddy, ax, ay, J);
                    axs += ax;
                    ays += ay;
                    const int np = lens_np(code);
                    for (int k = 0; k < np; ++k) {
                        dA[0][lp + k] = J[0][k];
                        dA[1][lp + k] = J[1][k];
                    }
                    lp += np;
                }
                axs *= alpha_scaling;
                ays *= alpha_scaling;
                // sources at beta; G = sum_k (-alpha_scaling s_k) grad_beta I_k
                T Gx = T(0), Gy = T(0);
                for (int k = 0; k < st.n_src; ++k) {
                    const int pp = st.n_lens + k;
                    const T* r = trec + pp * REC_D;
                    const T sc = (T)st.src_scale[k];
                    T Iv, gx, gy, dI[7], ddx, ddy;
                    off(pp, ddx, ddy);
                    const T bdx = ddx - sc * axs, bdy = ddy - sc * ays;
                    sersic_grad(st.src[k], r, P + st.src_off[k], bdx, bdy, Iv, gx, gy, dI);
                    const int np = st.src[k] == LENSGB_LIGHT_SERSIC_ELLIPSE ? 7 : 5;
                    for (int j = 0; j < np; ++j) tgt[st.src_off[k] + j] += w * dI[j];
                    Gx -= alpha_scaling * sc * gx;
                    Gy -= alpha_scaling * sc * gy;
                    if (mode == GRAD_FLAG_PASS && Iv > T(0)) {
                        // relative error of d I / d beta from the FP32 error of beta
                        const T xp = r[7] * bdx + r[8] * bdy, yp = r[9] * bdx + r[10] * bdy;
                        const T R = fmax(sqrt(xp * xp + yp * yp), T(0.0001));
                        const T gl_ = sqrt(gx * gx + gy * gy) / Iv;
                        const T pred = (gl_ + T(1) / R) * (T)GRAD_KAPPA * sc *
                                       (fabs(axs) + fabs(ays));
                        ill |= pred > (T)tau;
                    }
                }
                for (int c = 0; c < lp; ++c)
                    tgt[st.lens_off[0] + c] += w * (Gx * dA[0][c] + Gy * dA[1][c]);
                // lens light at theta
                for (int k = 0; k < st.n_ll; ++k) {
                    const int pp = st.n_lens + st.n_src + k;
                    const T* r = trec + pp * REC_D;
                    T Iv, gx, gy, dI[7], ddx, ddy;
                    off(pp, ddx, ddy);
                    sersic_grad(st.ll[k], r, P + st.ll_off[k], ddx, ddy, Iv, gx, gy, dI);
                    const int np = st.ll[k] == LENSGB_LIGHT_SERSIC_ELLIPSE ? 7 : 5;
                    for (int j = 0; j < np; ++j) tgt[st.ll_off[k] + j] += w * dI[j];
                }
            }
        }
        if (mode == GRAD_FLAG_PASS) {
            if (ill)
                flag[(long long)inst * npix + pix] = 1;  // the FP64 pass takes this pixel
            else
                for (int k = 0; k < NP; ++k) acc[k] += pacc[k];
        }
    }
    // fixed-order block reduction, one parameter at a time
    __shared__ double red[GRAD_THREADS];
    double* out = partial + ((long long)inst * gridDim.x + blockIdx.x) * NP;
    for (int k = 0; k < NP; ++k) {
        red[threadIdx.x] = (double)acc[k];
        __syncthreads();
        for (int s2 = GRAD_THREADS / 2; s2 > 0; s2 >>= 1) {
            if (threadIdx.x < s2) red[threadIdx.x] += red[threadIdx.x + s2];
            __syncthreads();
        }
        if (threadIdx.x == 0) out[k] = red[0];
        __syncthreads();
    }
}

// Sums the per-CTA partials in a fixed order; partial2 (or null): the partials
// of the FP64 pass over flagged pixels, added after the first set.
__global__ void grad_reduce_kernel(const double* __restrict__ partial,
                                   const double* __restrict__ partial2, int n_chunks, int NP,
                                   int n_inst, double* __restrict__ grad) {
    const int gid = blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= n_inst * NP) return;
    const int inst = gid / NP, k = gid % NP;
    double s = 0.0;
    for (int c = 0; c < n_chunks; ++c) s += partial[((long long)inst * n_chunks + c) * NP + k];
    if (partial2) {
        double s2 = 0.0;
        for (int c = 0; c < n_chunks; ++c)
            s2 += partial2[((long long)inst * n_chunks + c) * NP + k];
        s += s2;
    }
    grad[gid] = s;
}

int grad_chunks(const GridDesc& g) {
    const long long npix = (long long)g.nx * g.ny;
    return (int)((npix + GRAD_THREADS * GRAD_PPT - 1) / (GRAD_THREADS * GRAD_PPT));
}

bool grad_supported(const StackDesc& st) {
    if (st.n_params > GRAD_MAXP) return false;
    int lp = 0;
    for (int p = 0; p < st.n_lens; ++p) {
        const int np = lens_np(st.lens[p]);
        if (np == 0) return false;
        lp += np;
        if (p > 0 && st.lens_off[p] != st.lens_off[p - 1] + lens_np(st.lens[p - 1])) return false;
    }
    return lp <= GRAD_MAX_LENSP;
}

int launch_grad_weights(const double* image, int n_inst, long long npix, const LoglikeArgs& la,
                        double* gm, double* logl, cudaStream_t stream) {
    if (n_inst <= 0) return 0;
    loglike_weights_kernel<<<n_inst, 256, 0, stream>>>(image, npix, la, gm, logl);
    return 0;
}

// Edge padding as an explicit (ny + 2h) x (nx + 2h) image: pad[p][q] =
// in[clamp(p - h)][clamp(q - h)].  Its transpose folds the halo back onto the
// edge pixels: fold_edge_kernel sums, for each pixel, the padded pixels that
// clamp to it (its own, plus the halo rows / columns beyond an edge).
__global__ void embed_pad_kernel(const double* __restrict__ in, double* __restrict__ pad,
                                 int n_inst, int ny, int nx, int h) {
    const int PW = nx + 2 * h, PH = ny + 2 * h;
    const long long per = (long long)PW * PH;
    const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= per * n_inst) return;
    const long long inst = gid / per, e = gid - inst * per;
    const int r = (int)(e / PW) - h, c = (int)(e % PW) - h;
    pad[gid] = (r >= 0 && r < ny && c >= 0 && c < nx) ? in[(inst * ny + r) * nx + c] : 0.0;
}

__global__ void fold_edge_kernel(const double* __restrict__ pad, double* __restrict__ out,
                                 int n_inst, int ny, int nx, int h) {
    const long long per = (long long)nx * ny;
    const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= per * n_inst) return;
    const long long inst = gid / per, e = gid - inst * per;
    const int row = (int)(e / nx), col = (int)(e % nx);
    const int PW = nx + 2 * h, PH = ny + 2 * h;
    const int r0 = row == 0 ? 0 : row + h, r1 = row == ny - 1 ? ny - 1 + 2 * h : row + h;
    const int c0 = col == 0 ? 0 : col + h, c1 = col == nx - 1 ? nx - 1 + 2 * h : col + h;
    const double* p = pad + inst * (long long)PW * PH;
    double acc = 0.0;
    for (int r = r0; r <= r1; ++r)
        for (int c = c0; c <= c1; ++c) acc += p[(long long)r * PW + c];
    out[gid] = acc;
}

int launch_conv_transpose(const double* in, double* out, const double* psf, long long psf_stride,
                          int K, int edge, int n_inst, int ny, int nx, double* psf_flip,
                          double* pad_a, double* pad_b, cudaStream_t stream) {
    if (n_inst <= 0) return 0;
    const long long kk = (long long)K * K;
    const long long nk = kk * n_inst;
    flip_psf_kernel<<<(unsigned)((nk + 255) / 256), 256, 0, stream>>>(psf, psf_flip, K, psf_stride,
                                                                       n_inst);
    if (!edge)
        return launch_conv(in, out, psf_flip, kk, n_inst, ny, nx, K, 0, LENSGB_FP64, stream);
    // edge padding: out = fold(conv_zero(pad(in)))
    const int h = K / 2;
    const long long np = (long long)(ny + 2 * h) * (nx + 2 * h) * n_inst;
    embed_pad_kernel<<<(unsigned)((np + 255) / 256), 256, 0, stream>>>(in, pad_a, n_inst, ny, nx,
                                                                        h);
    if (launch_conv(pad_a, pad_b, psf_flip, kk, n_inst, ny + 2 * h, nx + 2 * h, K, 0, LENSGB_FP64,
                    stream))
        return -1;
    const long long n = (long long)ny * nx * n_inst;
    fold_edge_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(pad_b, out, n_inst, ny, nx,
                                                                       h);
    return 0;
}

__global__ void crop_kernel(const double* __restrict__ full, double* __restrict__ sub, int n_inst,
                            int n, int r0, int c0, int ny_full, int nx_full) {
    const long long per = (long long)n * n;
    const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= per * n_inst) return;
    const long long inst = gid / per, e = gid - inst * per;
    const int r = (int)(e / n), c = (int)(e % n);
    sub[gid] = full[(inst * ny_full + r0 + r) * (long long)nx_full + c0 + c];
}

int launch_crop(const double* full, double* sub, int n_inst, int n, int r0, int c0, int ny_full,
                int nx_full, cudaStream_t stream) {
    const long long total = (long long)n * n * n_inst;
    if (total <= 0) return 0;
    crop_kernel<<<(unsigned)((total + 255) / 256), 256, 0, stream>>>(full, sub, n_inst, n, r0, c0,
                                                                      ny_full, nx_full);
    return 0;
}

// hr (n_inst x ny*s x nx*s) = or += low (n_inst x ny x nx) x scale, each pixel
// spread over its s x s block: the transpose of the block mean (times scale s^2).
__global__ void expand_kernel(const double* __restrict__ low, double* __restrict__ hr,
                              int n_inst, int ny, int nx, int s, double scale, int accumulate) {
    const long long W = (long long)nx * s, per = W * ny * s;
    const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= per * n_inst) return;
    const long long inst = gid / per, e = gid - inst * per;
    const int r = (int)(e / W) / s, c = (int)(e % W) / s;
    const double v = low[(inst * ny + r) * (long long)nx + c] * scale;
    hr[gid] = accumulate ? hr[gid] + v : v;
}

int launch_expand(const double* low, double* hr, int n_inst, int ny, int nx, int s, double scale,
                  int accumulate, cudaStream_t stream) {
    const long long total = (long long)ny * nx * s * s * n_inst;
    if (total <= 0) return 0;
    expand_kernel<<<(unsigned)((total + 255) / 256), 256, 0, stream>>>(low, hr, n_inst, ny, nx, s,
                                                                        scale, accumulate);
    return 0;
}

__global__ void scale_kernel(double* __restrict__ x, long long n, double a) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] *= a;
}

int launch_scale(double* x, long long n, double a, cudaStream_t stream) {
    if (n <= 0) return 0;
    scale_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(x, n, a);
    return 0;
}

int launch_grad_rays(const GridDesc& g, const StackDesc& st, int n_inst, const double* params,
                     const double* rec_d, const double* coef_d, double* dcoef, const double* gl,
                     double w_scale, double* partial, double* grad, int precision,
                     unsigned char* flag, float tau, cudaStream_t stream) {
    if (n_inst <= 0) return 0;
    if (st.n_lens > 0) {
        // one warp per CTA: FP64 recurrences, spread over as many SMs as possible
        const int n = n_inst * st.n_lens;
        epl_dcoef_kernel<<<(n + 31) / 32, 32, 0, stream>>>(st, n_inst, rec_d, coef_d, dcoef);
    }
    const int chunks = grad_chunks(g);
    const int n_prof = st.n_lens + st.n_src + st.n_ll;
    const size_t nd = (size_t)(n_prof * REC_D + 2 * st.n_epl * EPL_NMAX);
    const dim3 grid((unsigned)chunks, (unsigned)n_inst);
    const size_t smem64 = nd * sizeof(double);
    if (smem64 > 48 * 1024)
        cudaFuncSetAttribute(grad_ray_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem64);
    double* partial2 = nullptr;
    if (precision == LENSGB_FP64) {
        grad_ray_kernel<double><<<grid, GRAD_THREADS, smem64, stream>>>(
            g, st, params, rec_d, coef_d, dcoef, gl, w_scale, partial, nullptr, 0.f, GRAD_ALL);
    } else {
        // the FP64 arrays, then their FP32 copies and the FP32 parameter row
        const size_t smem = nd * sizeof(double) + (nd + (size_t)st.n_params) * sizeof(float);
        if (smem > 48 * 1024)
            cudaFuncSetAttribute(grad_ray_kernel<float>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        const long long npix = (long long)g.nx * g.ny;
        if (cudaMemsetAsync(flag, 0, (size_t)n_inst * npix, stream) != cudaSuccess) return -1;
        partial2 = partial + (size_t)n_inst * chunks * st.n_params;
        grad_ray_kernel<float><<<grid, GRAD_THREADS, smem, stream>>>(
            g, st, params, rec_d, coef_d, dcoef, gl, w_scale, partial, flag, tau,
            GRAD_FLAG_PASS);
        grad_ray_kernel<double><<<grid, GRAD_THREADS, smem64, stream>>>(
            g, st, params, rec_d, coef_d, dcoef, gl, w_scale, partial2, flag, tau,
            GRAD_ONLY_FLAGGED);
    }
    const int n = n_inst * st.n_params;
    grad_reduce_kernel<<<(n + 127) / 128, 128, 0, stream>>>(partial, partial2, chunks,
                                                           st.n_params, n_inst, grad);
    return 0;
}

// LensModel.hessian (LensModel/lens_model.py:384-414 -> single_plane.py:142-180):
// f_xx, f_xy, f_yx, f_yy of the lens stack at n points, the derivatives of each
// profile's deflection with respect to the ray position taken from the same
// dual-number evaluation as the adjoint (the centre derivatives, negated), times
// alpha_scaling.  One thread per point; n_per points per system (parameter
// row); out holds the four components as four consecutive arrays of n.
__global__ void hessian_points_kernel(StackDesc st, const double* __restrict__ rec,
                                      const double* __restrict__ coef,
                                      const double* __restrict__ params,
                                      const double* __restrict__ x, const double* __restrict__ y,
                                      double* __restrict__ out, long long n, long long n_per) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const long long inst = i / n_per;
    const double X = x[i], Y = y[i];
    const double* P = params + inst * st.n_params;
    const double* rec_i = rec + inst * st.n_lens * REC_D;
    const double* coef_i = coef ? coef + inst * st.n_epl * EPL_NMAX : nullptr;
    double h[4] = {0.0, 0.0, 0.0, 0.0};
    for (int p = 0; p < st.n_lens; ++p) {
        const int code = st.lens[p];
        const double* r = rec_i + p * REC_D;
        const double* a = P + st.lens_off[p];
        const double dx = X - r[RD_CX], dy = Y - r[RD_CY];
        if (code == LENSGB_LENS_CONVERGENCE) {
            h[0] += r[2];
            h[3] += r[2];
            continue;
        }
        double ax, ay, J[2][GJ];
        int co;
        if (code == LENSGB_LENS_EPL || code == LENSGB_LENS_EPL_MULTIPOLE_M1M3M4) {
            // dF/dt enters only the t direction of the duals: the coefficient table
            // stands in for it
            const double* F = coef_i + st.epl_slot[p] * EPL_NMAX;
            if (code == LENSGB_LENS_EPL)
                epl_alpha_grad(r, F, F, a, dx, dy, ax, ay, J);
            else
                multipole_alpha_grad(r, F, F, a, dx, dy, ax, ay, J);
            co = 4;
        } else if (code == LENSGB_LENS_NFW_ELLIPSE_CSE) {
            cse_alpha_grad(r, a, dx, dy, ax, ay, J);
            co = 4;
        } else if (code == LENSGB_LENS_SIE || code == LENSGB_LENS_NIE) {
            nie_alpha_grad(code, r, a, dx, dy, ax, ay, J);
            co = code == LENSGB_LENS_SIE ? 3 : 4;
        } else if (code == LENSGB_LENS_NFW || code == LENSGB_LENS_TNFW) {
            nfw_alpha_grad(code, a, dx, dy, ax, ay, J);
            co = code == LENSGB_LENS_TNFW ? 3 : 2;
        } else {
            shear_alpha_grad(r, dx, dy, ax, ay, J);
            co = 2;
        }
        h[0] -= J[0][co];
        h[1] -= J[0][co + 1];
        h[2] -= J[1][co];
        h[3] -= J[1][co + 1];
    }
    for (int c = 0; c < 4; ++c) out[c * n + i] = h[c] * st.alpha_scaling;
}

bool hessian_supported(const StackDesc& st) {
    for (int p = 0; p < st.n_lens; ++p)
        if (st.lens[p] != LENSGB_LENS_CONVERGENCE && lens_np(st.lens[p]) <= 0) return false;
    return true;
}

int launch_hessian_points(const StackDesc& st, const double* rec, const double* coef,
                          const double* params, const double* x, const double* y, double* out,
                          long long n, long long n_per, cudaStream_t stream) {
    if (n <= 0 || n_per <= 0) return 0;
    const int threads = 128;
    hessian_points_kernel<<<(unsigned)((n + threads - 1) / threads), threads, 0, stream>>>(
        st, rec, coef, params, x, y, out, n, n_per);
    return 0;
}

}  // namespace lensgb

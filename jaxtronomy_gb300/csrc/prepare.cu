// Prepare kernel: converts each system's raw kwargs row into per-profile
// records (FP64 and FP32 copies) and the EPL series coefficient tables.
// One thread per (system, profile).  All arithmetic here is FP64.
//
// Parameter conversions follow (JAXtronomy source tree):
//   ellipticity2phi_q   Util/param_util.py:88-99
//   NIE._param_conv     LensModel/Profiles/nie.py:182-200, :255-272
//   EPL._param_conv     LensModel/Profiles/epl.py:111-124; nmax choice :311-319
//   F_n recurrence      Util/hyp2f1_util.py:156-166
//   NFW.alpha2rho0      LensModel/Profiles/nfw.py:386-395 (Rs floor :100)
//   SersicUtil.b_n      LensModel/Profiles/sersic_utils.py:69-80, floors :239-258
//   product average     Util/param_util.py:103-123
#include <math.h>

#include "cse_table.h"
#include "launch.h"
#include "profiles.cuh"

namespace lensgb {

__device__ static void ellip_phi_q(double e1, double e2, double& phi, double& q) {
    phi = atan2(e2, e1) / 2;
    double c = sqrt(e1 * e1 + e2 * e2);
    c = c < 0.9999 ? c : 0.9999;
    q = (1 - c) / (1 + c);
}

__device__ static int epl_nmax_of(double f) {
    if (f == 0) return 0;
    if (f < 0.12) return 10;
    if (f < 0.4) return 20;
    if (f < 0.6) return 35;
    if (f < 0.73) return 50;
    if (f < 0.86) return 100;
    if (f < 0.92) return 200;
    return 500;
}

// FP32 split of the offset between the supersampled ray (0,0) and a centre.
__device__ static void write_offsets(const GridDesc& g, double cx, double cy, float* f) {
    split_double(g.ra00 - cx, f[RF_X0H], f[RF_X0L]);
    split_double(g.dec00 - cy, f[RF_Y0H], f[RF_Y0L]);
}

// Record of lens profile `code` from its kwargs a[] (param_names order).  Fd/Ff
// receive the profile's coefficient table (EPL series F_n, CSE term constants)
// when it has one (else they may be null).  d[] must be zeroed by the caller.
__device__ void prepare_lens_record(int code, const double* a, double* d, double* Fd, float* Ff) {
    if (code == LENSGB_LENS_SIE || code == LENSGB_LENS_NIE) {
        double theta_E = a[0], e1 = a[1], e2 = a[2];
        double s_scale = code == LENSGB_LENS_SIE ? 0.0000000001 : a[3];
        int co = code == LENSGB_LENS_SIE ? 3 : 4;
        double phi, q;
        ellip_phi_q(e1, e2, phi, q);
        double theta_E_conv = theta_E / sqrt((1.0 + q * q) / (2.0 * q));
        double b = theta_E_conv * sqrt((1 + q * q) / 2);
        double s = s_scale / sqrt(q);
        double qc = q >= 1 ? 0.99999999 : q;   // NIEMajorAxis.derivatives clamp
        double sq = sqrt(1.0 - qc * qc);
        d[RD_CX] = a[co];
        d[RD_CY] = a[co + 1];
        d[2] = b; d[3] = s; d[4] = qc; d[5] = cos(phi); d[6] = sin(phi);
        d[7] = sq; d[8] = b / sq; d[9] = qc * qc; d[10] = qc * qc * s; d[11] = qc * qc * s * s;
    } else if (code == LENSGB_LENS_EPL || code == LENSGB_LENS_EPL_MULTIPOLE_M1M3M4) {
        double theta_E = a[0], gamma = a[1], e1 = a[2], e2 = a[3];
        double phi, q;
        ellip_phi_q(e1, e2, phi, q);
        double t = gamma - 1;
        double b = theta_E * sqrt(q);
        double fq = (1.0 - q) / (1.0 + q);
        int nmax = epl_nmax_of(fq);
        d[RD_CX] = a[4];
        d[RD_CY] = a[5];
        d[2] = b; d[3] = t; d[4] = q; d[5] = cos(phi); d[6] = sin(phi); d[7] = fq;
        d[8] = (double)nmax; d[9] = 2.0 / (1.0 + q) * pow(b, t);
        // FP32-path constants: q cos, q sin, f^2/4, f/2, -t/2
        d[10] = q * d[5]; d[11] = q * d[6];
        d[12] = 0.25 * fq * fq; d[13] = 0.5 * fq; d[14] = -0.5 * t;
        // F_0 = 1, F_1 = 1 - 2B/C, F_n = ((n-1) F_{n-2} - (2B-C) F_{n-1}) / (C+n-1)
        double B = t / 2.0, C = 2.0 - B;
        double fpp = 1.0, fp = 1.0 - 2.0 * B / C;
        if (nmax > 0) { Fd[0] = fpp; Ff[0] = (float)fpp; }
        if (nmax > 1) { Fd[1] = fp; Ff[1] = (float)fp; }
        for (int n = 2; n < nmax; ++n) {
            double fn = ((n - 1.0) * fpp - (2.0 * B - C) * fp) / (C + n - 1.0);
            Fd[n] = fn;
            Ff[n] = (float)fn;
            fpp = fp;
            fp = fn;
        }
        // FP32 series length: since |w| <= f/(2-f), the terms n >= k change the
        // sum by at most sum_{m>=k} |F_m| (f/(2-f))^m; stop once that bound is
        // below 2^-27 (under FP32 resolution), never beyond the reference's nmax.
        int n32 = nmax;
        if (nmax > 1) {
            const double wmax = fq / (2.0 - fq);
            double tail = 0.0, wp = pow(wmax, (double)(nmax - 1));
            for (int m = nmax - 1; m >= 1; --m) {
                tail += fabs(Fd[m]) * wp;
                if (tail > 7.450580596923828e-09) break;
                n32 = m;
                wp /= wmax;
            }
        }
        d[15] = (double)n32;
        if (code == LENSGB_LENS_EPL_MULTIPOLE_M1M3M4) {
            // multipoles m = 1, 3, 4 about the EPL centre, strengths a_m =
            // a{m}_a theta_E / sqrt(q), angles phi_m = phi + delta_phi_m
            // (epl_multipole_m1m3m4.py:495-535); m = 1 uses r_E = theta_E
            const double rescale = theta_E / sqrt(q);
            const double a1 = a[6] * rescale, p1 = phi + a[7];
            const double a3 = a[8] * rescale, p3 = phi + a[9];
            const double a4 = a[10] * rescale, p4 = phi + a[11];
            d[16] = a1 / 2; d[17] = cos(p1); d[18] = sin(p1); d[19] = log(theta_E);
            d[20] = a3 / (1.0 - 9.0); d[21] = cos(3 * p3); d[22] = sin(3 * p3);
            d[23] = a4 / (1.0 - 16.0); d[24] = cos(4 * p4); d[25] = sin(4 * p4);
            d[26] = p1; d[27] = a3; d[28] = p3; d[29] = a4; d[30] = p4; d[31] = theta_E;
        }
    } else if (code == LENSGB_LENS_NFW_ELLIPSE_CSE) {
        double Rs = a[0], alpha_Rs = a[1], e1 = a[2], e2 = a[3];
        double phi, q;
        ellip_phi_q(e1, e2, phi, q);
        double rho0 = alpha_Rs / (4.0 * Rs * Rs * (1.0 + log(1.0 / 2.0)));
        d[RD_CX] = a[4];
        d[RD_CY] = a[5];
        d[2] = Rs; d[3] = 1.0 / Rs; d[4] = q; d[5] = cos(phi); d[6] = sin(phi);
        d[7] = sqrt(q); d[8] = 4.0 * CSE_NFW_TERMS; d[9] = 4 * rho0 * Rs * Rs * Rs / Rs;
        d[10] = q * q; d[11] = 1.0 - q * q;
        // per-term constants of the FP32 path, one float4 per term:
        // (q^2 s^2, s, q^2 s, a/s)
        double* Cd = Fd;
        float* Cf = Ff;
        for (int k = 0; k < CSE_NFW_TERMS; ++k) {
            const double s = kCseNfwS[k], ak = kCseNfwA[k];
            const double v[4] = {q * q * s * s, s, q * q * s, ak / s};
            for (int j = 0; j < 4; ++j) {
                Cd[4 * k + j] = v[j];
                Cf[4 * k + j] = (float)v[j];
            }
        }
    } else if (code == LENSGB_LENS_SHEAR) {
        d[RD_CX] = a[2];
        d[RD_CY] = a[3];
        d[2] = a[0]; d[3] = a[1];
    } else if (code == LENSGB_LENS_CONVERGENCE) {
        d[RD_CX] = a[1];
        d[RD_CY] = a[2];
        d[2] = a[0];
        d[3] = a[0] - (double)(float)a[0];
    } else if (code == LENSGB_LENS_NFW) {
        double Rs = a[0], alpha_Rs = a[1];
        double rho0 = alpha_Rs / (4.0 * Rs * Rs * (1.0 + log(1.0 / 2.0)));
        double Rsf = Rs < 0.0000001 ? 0.0000001 : Rs;
        d[RD_CX] = a[2];
        d[RD_CY] = a[3];
        d[2] = Rsf; d[3] = rho0; d[4] = 4 * rho0 * Rsf; d[5] = 1.0 / Rsf;
    } else if (code == LENSGB_LENS_TNFW) {
        double Rs = a[0], alpha_Rs = a[1], r_trunc = a[2];
        double rho0 = alpha_Rs / (4.0 * Rs * Rs * (1.0 + log(1.0 / 2.0)));
        d[RD_CX] = a[3];
        d[RD_CY] = a[4];
        const double tau = r_trunc / Rs;
        d[2] = Rs; d[3] = rho0; d[4] = tau; d[5] = 4 * rho0 * Rs; d[6] = 1.0 / Rs;
        // many-deflector FP32 constants: 1/tau, tau^2/(tau^2+1)^2, tau^2 - 1
        d[7] = 1.0 / tau; d[8] = tau * tau / ((tau * tau + 1) * (tau * tau + 1));
        d[9] = tau * tau - 1;
        // Outside x = s, s = max(tau, 1): the bracket b(x) of g(x) as a polynomial
        // in t = 2 s/x - 1 in [-1, 1], the Chebyshev interpolant at the TNFW_NC
        // nodes t_j = cos(pi (j + 1/2) / TNFW_NC) (within 1.3e-9 relative of b for
        // tau in [0.05, 300]), stored as monomial coefficients of t (their absolute
        // values sum to below 2 b, so Horner's rule in FP32 stays within ~1e-7).
        // Layout: d10 s^2, d11 4 rho0 Rs tau^2/(tau^2+1)^2, d12 2 s, d14.. the
        // coefficients (float slots 16..: 16-byte aligned for vector loads).
        const double sc = tau > 1.0 ? tau : 1.0;
        double ch[TNFW_NC];
        for (int k = 0; k < TNFW_NC; ++k) ch[k] = 0.0;
        for (int j = 0; j < TNFW_NC; ++j) {
            const double t = cospi((j + 0.5) / TNFW_NC);
            const double f = tnfw_bracket_d(2.0 * sc / (1.0 + t), tau) * (2.0 / TNFW_NC);
            double Tm = 1.0, T = t;  // T_{k-2}(t), T_{k-1}(t)
            ch[0] += 0.5 * f;
            ch[1] += f * t;
            for (int k = 2; k < TNFW_NC; ++k) {
                const double Tn = 2.0 * t * T - Tm;
                Tm = T;
                T = Tn;
                ch[k] += f * Tn;
            }
        }
        // sum_k ch_k T_k(t) in powers of t (T_k = 2 t T_{k-1} - T_{k-2})
        double Pm[TNFW_NC], P[TNFW_NC], mono[TNFW_NC];
        for (int k = 0; k < TNFW_NC; ++k) Pm[k] = P[k] = mono[k] = 0.0;
        Pm[0] = 1.0;
        P[1] = 1.0;
        mono[0] = ch[0];
        mono[1] = ch[1];
        for (int n = 2; n < TNFW_NC; ++n) {
            for (int k = TNFW_NC - 1; k >= 0; --k) {
                const double pn = (k > 0 ? 2.0 * P[k - 1] : 0.0) - Pm[k];
                Pm[k] = P[k];
                P[k] = pn;
                mono[k] += ch[n] * pn;
            }
        }
        for (int k = 0; k < TNFW_NC; ++k) d[14 + k] = mono[k];
        d[10] = sc * sc;
        d[11] = d[5] * d[8];
        d[12] = 2.0 * sc;
    }
}

// Record of light profile `code` (SERSIC / SERSIC_ELLIPSE) from its kwargs a[].
__device__ void prepare_light_record(int code, const double* a, double* d) {
    // SERSIC / SERSIC_ELLIPSE
    double amp = a[0], R_sersic = a[1], n = a[2];
    double e1 = 0, e2 = 0, cx, cy;
    if (code == LENSGB_LIGHT_SERSIC_ELLIPSE) {
        e1 = a[3]; e2 = a[4]; cx = a[5]; cy = a[6];
    } else {
        cx = a[3]; cy = a[4];
    }
    R_sersic = R_sersic > 0 ? R_sersic : 0;          // sersic_ellipse.py:88
    double Rs_ = R_sersic > 0.0001 ? R_sersic : 0.0001;  // _R_stable
    double bn = 1.9992 * n - 0.3271;
    bn = bn > 0.00001 ? bn : 0.00001;
    double norm = sqrt(fabs(1 - e1 * e1 - e2 * e2));
    norm = norm > 0.000001 ? norm : 0.000001;
    d[RD_CX] = cx;
    d[RD_CY] = cy;
    d[2] = amp; d[3] = Rs_; d[4] = 1.0 / Rs_; d[5] = 1.0 / n; d[6] = bn;
    d[7] = (1 - e1) / norm; d[8] = -e2 / norm; d[9] = -e2 / norm; d[10] = (1 + e1) / norm;
    // FP32-path constants: log2(1/R_s), b_n log2(e), b_n / n
    d[11] = log2(1.0 / Rs_); d[12] = bn * 1.4426950408889634; d[13] = bn / n;
}

// FP32 copy of a record (float slot k + 2 mirrors double slot k >= 2).
__device__ void finish_record_f(const double* d, float* f) {
    for (int k = 2; k + F_OFF < REC_F && k < REC_D; ++k) f[k + F_OFF] = (float)d[k];
}

__global__ void prepare_kernel(GridDesc g, StackDesc st, const double* __restrict__ params,
                               int n_inst, double* __restrict__ rec_d, float* __restrict__ rec_f,
                               double* __restrict__ coef_d, float* __restrict__ coef_f,
                               const GridDesc* __restrict__ grids, const int* __restrict__ n_dev) {
    const int n_prof = st.n_lens + st.n_src + st.n_ll;
    if (n_dev) n_inst = min(n_inst, *n_dev);
    long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (long long)n_inst * n_prof) return;
    const int inst = (int)(gid / n_prof);
    const int p = (int)(gid % n_prof);
    const double* P = params + (long long)inst * st.n_params;
    double* d = rec_d + ((long long)inst * n_prof + p) * REC_D;
    float* f = rec_f + ((long long)inst * n_prof + p) * REC_F;
    for (int k = 0; k < REC_D; ++k) d[k] = 0.0;

    int kind, code, off;
    if (p < st.n_lens) {
        kind = 0; code = st.lens[p]; off = st.lens_off[p];
    } else if (p < st.n_lens + st.n_src) {
        kind = 1; code = st.src[p - st.n_lens]; off = st.src_off[p - st.n_lens];
    } else {
        kind = 2; code = st.ll[p - st.n_lens - st.n_src]; off = st.ll_off[p - st.n_lens - st.n_src];
    }
    const double* a = P + off;

    if (kind == 0) {
        const int slot_e = st.epl_slot[p];
        double* Fd = slot_e >= 0 ? coef_d + ((long long)inst * st.n_epl + slot_e) * EPL_NMAX : nullptr;
        float* Ff = slot_e >= 0 ? coef_f + ((long long)inst * st.n_epl + slot_e) * EPL_NMAX : nullptr;
        prepare_lens_record(code, a, d, Fd, Ff);
    } else {
        prepare_light_record(code, a, d);
    }
    finish_record_f(d, f);
    write_offsets(grids ? grids[inst] : g, d[RD_CX], d[RD_CY], f);
}

int launch_prepare(const GridDesc& g, const StackDesc& st, const double* params, int n_inst,
                   double* rec_d, float* rec_f, double* coef_d, float* coef_f,
                   cudaStream_t stream, const GridDesc* grids, const int* n_dev) {
    const int n_prof = st.n_lens + st.n_src + st.n_ll;
    long long n = (long long)n_inst * n_prof;
    if (n == 0) return 0;
    // one warp per CTA: each thread's FP64 set-up (EPL tables, transcendentals)
    // runs on GB300's FP64 units at 1/64 of the FP32 rate, so the threads are
    // spread over as many SMs as possible rather than packed four warps per SM
    int threads = 32;
    int blocks = (int)((n + threads - 1) / threads);
    prepare_kernel<<<blocks, threads, 0, stream>>>(g, st, params, n_inst, rec_d, rec_f, coef_d,
                                                   coef_f, grids, n_dev);
    return 0;
}

}  // namespace lensgb

namespace lensgb {

// Bound on |alpha| of one deflector, the quantity that decides whether its
// terms may run in FP32 (deflection scale theta_E of the power laws; NFW-type
// deflections peak near 1.01 alpha_Rs, doubled for ellipticity).  SHEAR and
// CONVERGENCE grow without bound away from their origin and run in FP64 in
// single-plane calls (the multi-plane kernel evaluates CONVERGENCE as an
// FP32-pair product instead).
__device__ static double bulk_alpha_bound(int code, const double* a) {
    switch (code) {
        case LENSGB_LENS_SIE:
        case LENSGB_LENS_NIE:
        case LENSGB_LENS_EPL:
        case LENSGB_LENS_EPL_MULTIPOLE_M1M3M4: return fabs(a[0]);
        case LENSGB_LENS_NFW:
        case LENSGB_LENS_TNFW:
        case LENSGB_LENS_NFW_ELLIPSE_CSE: return 2.0 * fabs(a[1]);
        default: return INFINITY;
    }
}

// One thread per deflector of a bulk call (SinglePlaneBulk.ray_shooting,
// single_plane_bulk.py:109-131): index -> profile code with lax.switch's
// clamping of out-of-range indices, record, coefficient table, and the
// deflector's tag (code | precision flag) for the ray kernel.
__global__ void bulk_prepare_kernel(BulkUnique u, const int* __restrict__ index,
                                    const double* __restrict__ params, int n_defl,
                                    double fp32_alpha_max, int* __restrict__ tag,
                                    double* __restrict__ rec_d, float* __restrict__ rec_f,
                                    double* __restrict__ coef_d, float* __restrict__ coef_f) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_defl) return;
    int k = index[i];
    k = k < 0 ? 0 : (k > u.n ? u.n : k);  // slot u.n is the NULL profile
    const int code = k < u.n ? u.code[k] : LENSGB_LENS_NULL;
    const double* a = params + (long long)i * LENSGB_BULK_PARAM_STRIDE;
    double* d = rec_d + (long long)i * REC_D;
    float* f = rec_f + (long long)i * REC_F;
    for (int j = 0; j < REC_D; ++j) d[j] = 0.0;
    double* Fd = coef_d ? coef_d + (long long)i * EPL_NMAX : nullptr;
    float* Ff = coef_f ? coef_f + (long long)i * EPL_NMAX : nullptr;
    if (code != LENSGB_LENS_NULL) prepare_lens_record(code, a, d, Fd, Ff);
    finish_record_f(d, f);
    // FP32 split of the centre: x - c = (x_hi - c_hi) + (x_lo - c_lo) is then
    // accurate to FP32 precision relative to the offset itself
    split_double(d[RD_CX], f[RF_X0H], f[RF_X0L]);
    split_double(d[RD_CY], f[RF_Y0H], f[RF_Y0L]);
    int t = code;
    if (code != LENSGB_LENS_NULL && !(bulk_alpha_bound(code, a) <= fp32_alpha_max))
        t |= BULK_TAG_FP64;
    tag[i] = t;
}

int launch_bulk_prepare(const BulkUnique& u, const int* index, const double* params, int n_defl,
                        double fp32_alpha_max, int* tag, double* rec_d, float* rec_f,
                        double* coef_d, float* coef_f, cudaStream_t stream) {
    if (n_defl <= 0) return 0;
    // one warp per CTA, spreading the FP64 set-up (the TNFW bracket polynomial's
    // 12 closed-form evaluations per deflector) over as many SMs as possible
    const int threads = 32;
    bulk_prepare_kernel<<<(n_defl + threads - 1) / threads, threads, 0, stream>>>(
        u, index, params, n_defl, fp32_alpha_max, tag, rec_d, rec_f, coef_d, coef_f);
    return 0;
}

}  // namespace lensgb
